// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k1_m1_b1_dna16_fe0, 1, run_gaps, 1, 1, 0, 0, false, false, false, false, int16_t, Dna5, false)
SEQAN_REF_UNIT(k2_m0_b0_dna32_fe0, 2, run_segments, 0, 0, 1, 0, false, false, false, false, int32_t, Dna5, false)
