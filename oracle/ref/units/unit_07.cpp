// Instantiation unit: a few reference call shapes, built in parallel (see ref_common.h).
#include "../ref_common.h"

SEQAN_REF_UNIT(k0_m1_b0_aa16_fe0, 0, run_score, 1, 0, 2, 0, false, false, false, false, int16_t, AminoAcid, true)
SEQAN_REF_UNIT(k0_m0_b1_dna16_fe0, 0, run_score, 0, 1, 0, 0, false, false, false, false, int16_t, Dna5, false)
