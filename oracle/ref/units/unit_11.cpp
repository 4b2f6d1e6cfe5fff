// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k1_m0_b0_dna16_fe9, 1, run_gaps, 0, 0, 0, 9, true, false, false, true, int16_t, Dna5, false)
SEQAN_REF_UNIT(k1_m0_b0_dna16_fe6, 1, run_gaps, 0, 0, 0, 6, false, true, true, false, int16_t, Dna5, false)
