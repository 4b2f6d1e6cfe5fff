// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k2_m0_b0_dna32_fe13, 2, run_segments, 0, 0, 1, 13, true, false, true, true, int32_t, Dna5, false)
SEQAN_REF_UNIT(k2_m0_b0_dna32_fe14, 2, run_segments, 0, 0, 1, 14, false, true, true, true, int32_t, Dna5, false)
