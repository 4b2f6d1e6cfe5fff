// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k1_m0_b0_aa16_fe6, 1, run_gaps, 0, 0, 2, 6, false, true, true, false, int16_t, AminoAcid, true)
SEQAN_REF_UNIT(k1_m1_b0_aa16_fe0, 1, run_gaps, 1, 0, 2, 0, false, false, false, false, int16_t, AminoAcid, true)
