// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k1_m0_b0_aa16_fe15, 1, run_gaps, 0, 0, 2, 15, true, true, true, true, int16_t, AminoAcid, true)
SEQAN_REF_UNIT(k1_m0_b0_aa16_fe9, 1, run_gaps, 0, 0, 2, 9, true, false, false, true, int16_t, AminoAcid, true)
