/* TEST INFRASTRUCTURE ONLY (reference oracle).
 *
 * The five alignment_t helpers that bwt.c calls, written to behave like
 * c/src/bioformats/bam/alignment.c:7-42 (alignment_new,
 * alignment_init_single_end), :253 (alignment_free) and :467-473
 * (is_/set_secondary_alignment).  The real alignment.c cannot be built here
 * because it needs the un-vendored samtools library.
 */
#include <stdlib.h>
#include "bioformats/bam/alignment.h"

alignment_t *alignment_new(void) { return (alignment_t *)calloc(1, sizeof(alignment_t)); }

void alignment_init_single_end(char *query_name, char *sequence, char *quality, short int strand,
                               unsigned int chromosome, int position, char *cigar,
                               short int num_cigar_operations, int map_quality, short int is_seq_mapped,
                               short int secondary_alignment, int optional_fields_length,
                               uint8_t *optional_fields, alignment_t *a) {
  a->query_name = query_name;
  a->sequence = sequence;
  a->quality = quality;
  a->cigar = cigar;
  a->chromosome = chromosome;
  a->position = position;
  a->mate_position = -1;
  a->mate_chromosome = -1;
  a->template_length = 0;
  a->map_quality = map_quality;
  a->num_cigar_operations = num_cigar_operations;
  a->is_paired_end = 0;
  a->is_paired_end_mapped = 0;
  a->is_seq_mapped = is_seq_mapped;
  a->is_mate_mapped = 0;
  a->seq_strand = strand;
  a->mate_strand = 0;
  a->pair_num = 0;
  a->secondary_alignment = secondary_alignment;
  a->fails_quality_check = 0;
  a->pc_optical_duplicate = 0;
  a->optional_fields = optional_fields;
  a->optional_fields_length = optional_fields_length;
  a->map_len = 0;
  a->alig_data = NULL;
}

void alignment_free(alignment_t *p) {
  if (!p) return;
  free(p->query_name);
  free(p->sequence);
  free(p->quality);
  free(p->cigar);
  free(p->optional_fields);
  free(p);
}

short int is_secondary_alignment(alignment_t *a) { return a->secondary_alignment; }
void set_secondary_alignment(short int set, alignment_t *a) { a->secondary_alignment = set; }
