// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k2_m1_b1_dna32_fe0, 2, run_segments, 1, 1, 1, 0, false, false, false, false, int32_t, Dna5, false)
SEQAN_REF_UNIT(k2_m1_b0_aa32_fe0, 2, run_segments, 1, 0, 3, 0, false, false, false, false, int32_t, AminoAcid, true)
