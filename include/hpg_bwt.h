/*
 * hpg_bwt.h -- drop-in C ABI of the GB300 FM-index read-mapping path.
 *
 * Replaces the FM-index mapping entry points of opencb/hpg-libs
 * (c/src/aligners/bwt/bwt.h).  Host code stays C: link libhpgbwt.so in place
 * of the bwt objects of libhpg.a.  The index lives in GPU memory; every
 * search runs as sm_103a CUDA kernels and there is no CPU fallback (without a
 * CUDA device, opening an index fails).
 *
 * The record types (bwt_optarg_t, bwt_index_t's leading fields, exome,
 * bwt_config_t) keep the reference's field layout so existing callers that
 * read them keep working.  bwt_index_t appends private fields after the
 * reference's ones.
 */
#ifndef HPG_BWT_H
#define HPG_BWT_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

#include "hpg_bwt_records.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ types ---- */

/* c/src/aligners/bwt/search/io.h:22-29 (chromosome table of the index). */
#ifndef _SEARCH_IO_
#define IDMAX 500
typedef struct {
  int max_chromosomes;
  char *chromosome; /* names, IDMAX bytes each */
  uintmax_t *start;
  uintmax_t *end;
  uintmax_t *offset; /* size + 1 entries */
  uintmax_t size;
} exome;
#endif

/* c/src/aligners/bwt/bwt_commons.h:20-32 */
#ifndef BWT_COMMONS_H
typedef struct {
  uint8_t *table;
  char *nucleotides;
  char *reverse;
  uint8_t nA;
  uint8_t AA, CC, GG, TT;
  bool inverse_sa;
  bool duplicate_strand;
} bwt_config_t;
#endif

/* c/src/aligners/bwt/bwt.h:256-261 */
typedef struct bwt_optarg {
  size_t num_errors;
  size_t num_threads;
  int filter_read_mappings;
  int filter_seed_mappings;
} bwt_optarg_t;

/* c/src/aligners/bwt/bwt.h:273-281.  The four bwt_index pointers are opaque
 * here (the reference's host tables are replaced by the GPU index). */
typedef struct hpg_bwt_view hpg_bwt_view_t;
typedef struct {
  exome *karyotype;
  bwt_config_t bwt_config;
  hpg_bwt_view_t *backward;
  hpg_bwt_view_t *forward;
  hpg_bwt_view_t *backward_rev;
  hpg_bwt_view_t *forward_rev;
  char *dirname;
  void *gpu_; /* private: GPU context */
} bwt_index_t;

/* ---------------------------------------------------- index + options -- */

/* bwt.h:283 (bwt.c:682-713).  Loads <dirname> (reference on-disk format) and
 * uploads it to the current CUDA device.  Like the reference, an unreadable
 * index ends the process with EXIT_FAILURE; bwt_index_open reports instead. */
bwt_index_t *bwt_index_new(const char *dirname, bool inverse_sa);

/* bwt.h:285 (bwt.c:717-740) */
void bwt_index_free(bwt_index_t *index);

/* Non-exiting form of bwt_index_new: NULL and a message in errbuf on error.
 * device < 0 selects the current CUDA device.  No reference counterpart. */
bwt_index_t *bwt_index_open(const char *dirname, bool inverse_sa, int device, char *errbuf, size_t errlen);

/* bwt.h:263-268 (bwt.c:435-447) */
bwt_optarg_t *bwt_optarg_new(const size_t num_errors, const size_t num_threads, const int filter_read_mappings,
                             const int filter_seed_mappings);
/* bwt.h:268 (bwt.c:449-453) */
void bwt_optarg_free(bwt_optarg_t *optarg);

/* bwt.h:287-289 (bwt.c:744-819): writes the reference on-disk index format,
 * byte for byte.  The suffix arrays are built on GPU 0 when one is visible
 * (prefix doubling with a device radix sort), else on the host (SA-IS); the
 * files are the same either way.  Ends the process on error, like the
 * reference. */
void bwt_generate_index_files(char *ref_file, char *output_dir, unsigned int s_ratio, bool duplicate_strand,
                              char *bases);

/* Status-returning builder (0 ok, -1 with errbuf), suffix arrays on the host.
 * No reference counterpart. */
int hpg_bwt_build_index(const char *ref_file, const char *output_dir, unsigned int s_ratio, int duplicate_strand,
                        const char *bases, char *errbuf, size_t errlen);
/* The same with the suffix arrays built on CUDA device `device` (-1: on the
 * host).  A 3.1 Gbp genome needs about 100 GB of device memory.  No reference
 * counterpart. */
int hpg_bwt_build_index_on(const char *ref_file, const char *output_dir, unsigned int s_ratio,
                           int duplicate_strand, const char *bases, int device, char *errbuf, size_t errlen);

/* ------------------------------------------------ GPU batch search ---- */

/* Pipeline forms of the batch search. */
#define HPG_BWT_FORM_PLAIN   0 /* one thread per read and strand, one launch per stage */
#define HPG_BWT_FORM_BATCHED 1 /* persistent work-queue kernel launched from a CUDA graph */

/* Batched GPU form of the reference's search layer: for every read, mode
 * HPG_BWT_MODE_SEARCH1 runs the four vector searches and
 * BWSearch1VectorHelper per strand exactly as bwt.c:1940-2002 (declared at
 * search/search.h:202-205), keeping at most max_results hits per strand
 * (results_list capacity), then locates every row of every hit with the
 * sampled suffix array (get_SA, search/runtime.h:87) and the karyotype
 * (bwt.c:2158-2166).  Mode HPG_BWT_MODE_EXACT runs BWExactSearchBackward on
 * both strands (search/search.h:9-36).
 *
 * Reads: seqs[offsets[i] .. offsets[i+1]) in ASCII, n_reads + 1 offsets.
 * Reads shorter than 3 bases, or with characters outside the index alphabet
 * (undefined in the reference), get no hits.
 * Output: host arrays allocated by the library (large ones page-locked and
 * reused across calls); release with bwt_gpu_result_free only.  Returns 0, or
 * -1 (see bwt_gpu_last_error). */
int bwt_gpu_search_batch(bwt_index_t *index, int mode, int form, const char *seqs, const uint64_t *offsets,
                         size_t n_reads, uint32_t max_results, hpg_result_set_t *out);
void bwt_gpu_result_free(hpg_result_set_t *out);
/* k-error block search of bwt_map_inexact_read_2 (bwt.c:2401-2470): the
 * search layer's BWSearchCPU (search/search.h:200, search/search.c:1171-1405)
 * per strand, '+' over (backward, forward) and '-' over (forward_rev,
 * backward_rev), with the fragment size max(len / 2, 30) -- one or two
 * fragments, one error -- and result lists of capacity max_results.
 * out: hits in rl_final order per (read, strand) and every row of every hit
 * located as bwt.c:2640-2650 (0-based positions; the locate limit applies);
 * rs_truncated bit 0 = a list of the search refused a result (full).
 * anchors (4 n_reads entries) and n_anchors (2 n_reads), either may be NULL:
 * the rl_anchor results of the search, anchors[2 * (2 * read + strand) + a]
 * for a < n_anchors[2 * read + strand].  Reads as bwt_gpu_search_batch (3 to
 * 32767 bases in the alphabet, others get nothing).  Release out with
 * bwt_gpu_result_free.  Returns 0, or -1 (see bwt_gpu_last_error). */
int bwt_gpu_block_search(bwt_index_t *index, const char *seqs, const uint64_t *offsets, size_t n_reads,
                         uint32_t max_results, hpg_result_set_t *out, hpg_block_anchor_t *anchors,
                         uint8_t *n_anchors);
/* Device time of the last bwt_gpu_block_search's search kernel(s), ms. */
float bwt_gpu_block_search_ms(bwt_index_t *index);

/* Device-resident form for callers that keep reads in GPU memory: d_seqs and
 * d_offsets are device pointers (offsets relative to d_seqs; total_bases =
 * d_offsets[n_reads], the bytes of d_seqs in use; max_len = longest read).  Results stay
 * on the device until the next call; sizes are returned in out (its pointer
 * fields are device pointers).  Copy them with bwt_gpu_copy_result. */
int bwt_gpu_search_device(bwt_index_t *index, int mode, int form, const uint8_t *d_seqs, const uint64_t *d_offsets,
                          size_t n_reads, uint64_t total_bases, uint32_t max_len, uint32_t max_results,
                          hpg_result_set_t *out);
int bwt_gpu_copy_result(bwt_index_t *index, const hpg_result_set_t *dev, hpg_hit_t *hits, hpg_loc_t *locs,
                        uint32_t *rs_count, uint8_t *rs_truncated);

/* The CUDA stream (cudaStream_t) every kernel of this index runs on. */
void *bwt_gpu_stream(bwt_index_t *index);
/* Device times (ms) of the last call: encode, search, finalize, locate and,
 * as a fifth value, the part of search spent in the drain launch. */
void bwt_gpu_stage_ms(bwt_index_t *index, float *out, int n);
/* Count touched 32-byte index sectors during searches (for roofline figures). */
void bwt_gpu_set_census(bwt_index_t *index, int on);
unsigned long long bwt_gpu_census(bwt_index_t *index);
/* Reads per internal chunk of the plain form (0 = automatic). */
void bwt_gpu_set_chunk(bwt_index_t *index, size_t reads);
/* Batched-form tuning: register bound (1 = compiler's choice, 10 (fused form
 * only), 12 or 16 resident 128-thread blocks per SM), resident blocks per SM actually
 * launched (0 = occupancy limit), change points per lane held in shared
 * memory (2, 4 or 8; more spill to the device queue; 0 = split form: a
 * chain-only kernel queues every change point for the drain launch; -1 =
 * lockstep form: one lane per read advances the read's four vector searches
 * together and queues change points), chains claimed per refill (1..8).  Setting
 * a tuning selects the fused, split or lockstep form; an index opens in the
 * warp-cooperative form (bwt_gpu_set_wave_group: 16 reads per warp group, one
 * launch per index direction, 12 blocks per SM).  get: {threads per block,
 * blocks per SM, stack depth (-2: warp-cooperative), chains per claim (reads
 * per warp group in the warp-cooperative form), register bound}. */
void bwt_gpu_set_tuning(bwt_index_t *index, int min_blocks, int blocks_per_sm, int stack_depth,
                        int chains_per_claim);
void bwt_gpu_get_tuning(bwt_index_t *index, int *out5);
/* How occurrence blocks are fetched by every kernel of this index: 0 two
 * 16-byte loads; 1 one 32-byte load; 2 one 32-byte load that bypasses L1 and
 * marks the line evict-last in L2 (default); 3 32-byte load, L2 hint only. */
void bwt_gpu_set_load_mode(bwt_index_t *index, int mode);
int bwt_gpu_load_mode(bwt_index_t *index);
/* Batched form launch: 1 (default) replays a CUDA graph captured once per
 * power-of-two read capacity (all sizes read from device memory, one host
 * synchronize per batch); 0 launches stage by stage with sizes read back to
 * the host between stages.  Results are identical. */
void bwt_gpu_set_graph(bwt_index_t *index, int on);
int bwt_gpu_graph(bwt_index_t *index);
/* With a chunk size set, bwt_gpu_search_batch of at least two chunks (batched
 * form, graph on) runs as a pipeline: chunk i+1's reads go in and chunk i-1's
 * records come out while chunk i is searched.  reads per chunk: 0 or SIZE_MAX
 * never (the default: on GB300 the copies slow the search by about their own
 * duration, so the overlap gains nothing). */
void bwt_gpu_set_pipeline_chunk(bwt_index_t *index, size_t reads);
/* Direction split of the batched search (fused form).  Every chain of a read
 * and its branches run on one index direction ('+' backward and '-' forward
 * on the backward index, the other two on the forward index).  0 (default):
 * any lane runs any chain; 1: SMs of the first half run the backward-index
 * chains and the other SMs the forward-index ones (a half that runs out takes
 * the other's reads); 2: one launch per direction, so the whole L2 holds one
 * direction's occurrence blocks at a time.  Results are identical. */
void bwt_gpu_set_direction_split(bwt_index_t *index, int mode);
int bwt_gpu_direction_split(bwt_index_t *index);
/* Warp-cooperative form of the batched search (no reference counterpart; the
 * reference's helper, search/search.c:1491-1709, runs one read per CPU
 * thread): 1..32 selects it, with that many reads claimed by a warp at a time
 * (32 / reads lanes per read); their bases are staged in shared memory, and
 * the warp's lanes share the group's chains and one stack of change points.
 * The direction split (0 or 2), register bound (1, 8 or 12 blocks per SM),
 * idle batch, start table and block-load form apply to it as to the fused
 * form.  0 returns to the fused form.  Results are identical. */
void bwt_gpu_set_wave_group(bwt_index_t *index, int reads);
/* Reads per warp group of the warp-cooperative form, 0 when another form is selected. */
int bwt_gpu_wave_group(bwt_index_t *index);
/* Wall time, in seconds, of the device pass of the last bwt_map_inexact_batch /
 * bwt_map_inexact_array_list / bwt_map_inexact_read call on this index: the
 * search, the row filter, the located rows, the 10 bp merge and the list order
 * (the rest of the call is the host's allocation of the records).  No
 * counterpart in the reference. */
double bwt_gpu_map_device_seconds(bwt_index_t *index);
/* Idle-lane batch of the batched search (fused form): a lane that finished its
 * work item waits, masked, until this many lanes of its warp have (or all
 * active ones have), and they take their next items together, so the code that
 * sets up a work item runs for many lanes at once.  1: each lane at once;
 * 8 by default (about 10 % faster on C2 than 1); up to 32.  Results are identical. */
void bwt_gpu_set_idle_batch(bwt_index_t *index, int lanes);
int bwt_gpu_idle_batch(bwt_index_t *index);
/* Locate limit of bwt_gpu_search_batch / _device and the serving form (no
 * counterpart in the reference's search layer, which locates every row; its
 * bwt_map_inexact_read drops repetitive strands with filter_read_mappings,
 * bwt.c:2148-2149, for the same reason).  A (read, strand) list whose kept
 * hits cover more than max_rows suffix-array rows keeps its hits but gets no
 * located rows, and bit 1 (value 2) of its rs_truncated entry is set.  Low-
 * complexity reads (a 50 bp read inside a homopolymer run of a 3 Gbp genome)
 * cover millions of rows each.  0, the default, locates every row. */
void bwt_gpu_set_locate_limit(bwt_index_t *index, uint64_t max_rows);
uint64_t bwt_gpu_locate_limit(bwt_index_t *index);
/* Start table of the batched search (fused and warp-cooperative forms): a
 * chain of a read of at least 2L+2 bases starts with one lookup of its first L
 * symbols in a table of 4^L intervals per index direction (8 MB each at L = 10)
 * instead of L dependent steps.  0 = no table (the default; the autotuner tries
 * 8, 10, 11, 12), at most 12.  Results are identical. */
int bwt_gpu_set_start_table(bwt_index_t *index, int symbols);
int bwt_gpu_start_table(bwt_index_t *index);
/* Autotuner: times the batched search on a device-resident read batch for
 * every candidate setting (60 fused, split and lockstep settings, then 12
 * warp-cooperative ones: 8, 16 or 32 reads per warp group x register bound 8
 * or 12 x direction split 0 or 2), keeps the fastest, then picks the fastest
 * block-load form for it (4 more runs), then the direction split (3 more, fused
 * form only), then the start-table length among 0, 8, 10, 11, 12 (5 more),
 * then the idle-lane batch among 1, 4, 8, 16 (4 more).  Optional table gets
 * rows of {min_blocks (or -1 - load mode, -50 - split, -100 - table length,
 * -200 - idle batch), blocks_per_sm, stack (-2: warp-cooperative),
 * chains_per_claim (reads per warp group), search us}. */
int bwt_gpu_autotune(bwt_index_t *index, const uint8_t *d_seqs, const uint64_t *d_offsets, size_t n_reads,
                     uint64_t total_bases, uint32_t max_len, uint32_t max_results, int *table, int max_rows,
                     int *rows);
/* Number of kernels this library has launched since it was loaded. */
unsigned long long bwt_gpu_launch_count(void);
/* Device bytes of the index's occurrence blocks (both directions). */
size_t bwt_gpu_index_bytes(bwt_index_t *index);
/* Measured ceiling of dependent random 32-byte sector reads over a buffer of
 * `bytes` on `device` (blocks x 128 threads, `steps` hops each), in sectors/s. */
int bwt_gpu_gather_ceiling(int device, size_t bytes, uint32_t blocks, uint32_t steps, double *sectors_per_s);
/* Message of the last failed call on this thread. */
const char *bwt_gpu_last_error(void);

/* ------------------------------------------- allocation-free search ---- */

/* No counterpart in the reference: an extra entry point of this library.
 *
 * BWSearch1 (both strands, as bwt_gpu_search_batch in mode
 * HPG_BWT_MODE_SEARCH1, without the locate step) for callers that must not
 * allocate device memory: processes whose HBM is owned by another allocator
 * (a serving runtime that has reserved the whole device for its own pool and
 * forbids side allocations), and latency-critical threads, where a
 * cudaMalloc/cudaFree can stall on device-wide synchronisation.  Its scratch
 * is one fixed 16 MiB array per device (bwt_gpu_noalloc_scratch_bytes()),
 * held until the process exits.  With CUDA's default lazy module loading the
 * runtime creates that array on the first call made on a device, so that
 * first call is the one that takes device memory: make it right after
 * bwt_index_new, before another allocator reserves the device's free memory
 * and before any stream capture.  Every later call allocates nothing.
 *
 * All buffers are the caller's device memory: d_seqs/d_offsets as in
 * bwt_gpu_search_device (max_len must cover the longest read; longer reads,
 * and reads whose offsets run backwards, get no hits); d_hits holds 2 * n_reads * max_results records,
 * hit i of (read r, strand s) at [(2*r + s) * max_results + i]; d_counts and
 * d_truncated hold 2 * n_reads entries.  The kernel is launched on `stream`
 * (the index's stream when NULL) and the call returns without waiting.
 *
 * Limit: n_reads * max(max_len, 3) may not exceed about 490 000 bases
 * (2 * n_reads * max_len * 17 bytes of scratch plus alignment); larger
 * batches are rejected with -1 and a message in
 * bwt_gpu_noalloc_last_error().  The scratch is fully rewritten before it is
 * read, so no call depends on what an earlier call left there, but every call
 * on a device shares it: calls whose kernels overlap on the GPU race and must
 * be serialised by the caller (one stream, or events).  The first call on a
 * device also looks up the scratch's device address (cudaGetSymbolAddress
 * with that device current).  Returns 0 once the kernel is queued; a runtime
 * error left pending by earlier work on the calling thread is not consumed. */
int bwt_gpu_search1_noalloc(bwt_index_t *index, const char *d_seqs, const uint64_t *d_offsets, size_t n_reads,
                            uint32_t max_len, uint32_t max_results, hpg_hit_t *d_hits, uint32_t *d_counts,
                            uint8_t *d_truncated, void *stream);
/* Size of the fixed scratch array, in bytes. */
size_t bwt_gpu_noalloc_scratch_bytes(void);
/* Message of the last failed bwt_gpu_search1_noalloc call on this thread. */
const char *bwt_gpu_noalloc_last_error(void);

/* ---- Serving form (no reference counterpart: the reference maps each batch
 * synchronously in the caller's thread, bwt.c:1097-1160).  A server owns the
 * index's stream until freed; other calls on that index meanwhile race.
 *
 * Requests of any size up to max_batch_reads / max_batch_bases are submitted
 * from any thread and mapped with BWSearch1 exactly as bwt_gpu_search_batch
 * maps them (HPG_BWT_MODE_SEARCH1, batched form, max_results per (read,
 * strand)): the result of a request is the same alone and in any mix.  A
 * worker thread admits waiting requests in arrival order while they fit the
 * batch capacity and the HBM budget (0 = a quarter of the device memory free
 * at creation), runs them as one graph replay, and forms the next batch from
 * new arrivals while a batch is on the GPU.  Creating a server frees the
 * index's batch-call workspaces and its graph plans above the batch capacity
 * (a device result of an earlier call is invalid after it, as after any call)
 * and captures the plans of every capacity class the server runs in.
 *
 * submit: the reads stay in the caller's memory (pinned memory copies fastest)
 * until wait returns for the ticket.  wait: 0 done, 1 timed out (timeout_ms
 * >= 0), -1 failed (bwt_gpu_last_error); `view` then points into the server's
 * pinned result buffers, read and hit ids relative to the request, valid until
 * release.  Unreleased requests hold their batch's buffers (three in turn).
 * stats: {batches, requests, reads, mean reads per batch, batch wall ms (sum),
 * pool regrowths, device bytes of the captured plans, HBM budget, largest
 * batch (reads), largest batch (requests), queued requests, hits per read,
 * rows per read}. */
typedef struct bwt_gpu_server bwt_gpu_server_t;
bwt_gpu_server_t *bwt_gpu_server_new(bwt_index_t *index, size_t max_batch_reads, uint64_t max_batch_bases,
                                     uint64_t hbm_budget_bytes, uint32_t max_results);
int bwt_gpu_server_submit(bwt_gpu_server_t *server, const char *seqs, const uint64_t *offsets, size_t n_reads,
                          uint64_t *ticket);
int bwt_gpu_server_wait(bwt_gpu_server_t *server, uint64_t ticket, hpg_result_set_t *view, double *latency_ms,
                        int timeout_ms);
int bwt_gpu_server_release(bwt_gpu_server_t *server, uint64_t ticket);
void bwt_gpu_server_stats(bwt_gpu_server_t *server, double *out, int n);
void bwt_gpu_server_free(bwt_gpu_server_t *server);

#ifdef __cplusplus
}
#endif

#endif /* HPG_BWT_H */
