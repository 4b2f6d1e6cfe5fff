// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k0_m0_b0_dna32_fe15, 0, run_score, 0, 0, 1, 15, true, true, true, true, int32_t, Dna5, false)
SEQAN_REF_UNIT(k0_m0_b0_dna32_fe9, 0, run_score, 0, 0, 1, 9, true, false, false, true, int32_t, Dna5, false)
