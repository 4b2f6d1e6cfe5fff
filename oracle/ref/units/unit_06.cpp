// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k0_m0_b0_aa16_fe9, 0, run_score, 0, 0, 2, 9, true, false, false, true, int16_t, AminoAcid, true)
SEQAN_REF_UNIT(k0_m0_b0_aa16_fe6, 0, run_score, 0, 0, 2, 6, false, true, true, false, int16_t, AminoAcid, true)
