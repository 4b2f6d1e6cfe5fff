// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k2_m0_b0_dna32_fe5, 2, run_segments, 0, 0, 1, 5, true, false, true, false, int32_t, Dna5, false)
SEQAN_REF_UNIT(k2_m0_b0_dna32_fe6, 2, run_segments, 0, 0, 1, 6, false, true, true, false, int32_t, Dna5, false)
