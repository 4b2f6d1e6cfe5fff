// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k1_m0_b1_dna16_fe9, 1, run_gaps, 0, 1, 0, 9, true, false, false, true, int16_t, Dna5, false)
SEQAN_REF_UNIT(k1_m0_b1_dna16_fe15, 1, run_gaps, 0, 1, 0, 15, true, true, true, true, int16_t, Dna5, false)
