// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k2_m0_b0_dna32_fe9, 2, run_segments, 0, 0, 1, 9, true, false, false, true, int32_t, Dna5, false)
SEQAN_REF_UNIT(k2_m0_b0_dna32_fe10, 2, run_segments, 0, 0, 1, 10, false, true, false, true, int32_t, Dna5, false)
