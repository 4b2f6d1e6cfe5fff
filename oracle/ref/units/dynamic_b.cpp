// DynamicGaps call shapes of the reference (see ../dynamic_common.h); kind 3 in the unit registry.
#include "../dynamic_common.h"

SEQAN_REF_UNIT(k3_m1_dna32_fe0, 3, run_dynamic, 1, 0, 1, 0, false, false, false, false, int32_t, Dna5, false)
SEQAN_REF_UNIT(k3_m0_dna16_fe0, 3, run_dynamic, 0, 0, 0, 0, false, false, false, false, int16_t, Dna5, false)
SEQAN_REF_UNIT(k3_m1_dna16_fe0, 3, run_dynamic, 1, 0, 0, 0, false, false, false, false, int16_t, Dna5, false)
SEQAN_REF_UNIT(k3_m1_aa16_fe0, 3, run_dynamic, 1, 0, 2, 0, false, false, false, false, int16_t, AminoAcid, true)
SEQAN_REF_UNIT(k3_m0_aa16_fe0, 3, run_dynamic, 0, 0, 2, 0, false, false, false, false, int16_t, AminoAcid, true)
