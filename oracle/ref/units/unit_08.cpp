// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k0_m0_b1_dna16_fe9, 0, run_score, 0, 1, 0, 9, true, false, false, true, int16_t, Dna5, false)
SEQAN_REF_UNIT(k0_m0_b1_dna32_fe0, 0, run_score, 0, 1, 1, 0, false, false, false, false, int32_t, Dna5, false)
