// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k0_m0_b0_aa16_fe0, 0, run_score, 0, 0, 2, 0, false, false, false, false, int16_t, AminoAcid, true)
SEQAN_REF_UNIT(k0_m0_b0_aa16_fe15, 0, run_score, 0, 0, 2, 15, true, true, true, true, int16_t, AminoAcid, true)
