// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k0_m0_b0_dna32_fe6, 0, run_score, 0, 0, 1, 6, false, true, true, false, int32_t, Dna5, false)
SEQAN_REF_UNIT(k0_m1_b0_dna32_fe0, 0, run_score, 1, 0, 1, 0, false, false, false, false, int32_t, Dna5, false)
