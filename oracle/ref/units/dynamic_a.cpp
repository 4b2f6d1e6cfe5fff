// DynamicGaps call shapes of the reference (see ../dynamic_common.h); kind 3 in the unit registry.
#include "../dynamic_common.h"

SEQAN_REF_UNIT(k3_m0_dna32_fe0, 3, run_dynamic, 0, 0, 1, 0, false, false, false, false, int32_t, Dna5, false)
SEQAN_REF_UNIT(k3_m0_dna32_fe15, 3, run_dynamic, 0, 0, 1, 15, true, true, true, true, int32_t, Dna5, false)
SEQAN_REF_UNIT(k3_m0_dna32_fe9, 3, run_dynamic, 0, 0, 1, 9, true, false, false, true, int32_t, Dna5, false)
SEQAN_REF_UNIT(k3_m0_dna32_fe6, 3, run_dynamic, 0, 0, 1, 6, false, true, true, false, int32_t, Dna5, false)
