// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k2_m0_b0_dna32_fe1, 2, run_segments, 0, 0, 1, 1, true, false, false, false, int32_t, Dna5, false)
SEQAN_REF_UNIT(k2_m0_b0_dna32_fe2, 2, run_segments, 0, 0, 1, 2, false, true, false, false, int32_t, Dna5, false)
