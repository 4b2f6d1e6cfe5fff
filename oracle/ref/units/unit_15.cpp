// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k1_m0_b0_dna32_fe0, 1, run_gaps, 0, 0, 1, 0, false, false, false, false, int32_t, Dna5, false)
SEQAN_REF_UNIT(k1_m0_b1_dna16_fe0, 1, run_gaps, 0, 1, 0, 0, false, false, false, false, int16_t, Dna5, false)
