/* Minimal stand-in for the un-vendored samtools header: the reference's
 * alignment.h only names these two types in prototypes the oracle never calls. */
#include <stdint.h>
typedef struct bam1_t bam1_t;
typedef struct bam_header_t bam_header_t;
