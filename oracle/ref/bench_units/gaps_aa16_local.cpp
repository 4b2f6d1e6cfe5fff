// Reference-arm instantiation: localAlignment(ExecutionPolicy<Parallel, Vectorial>, StringSet<Gaps>,
// StringSet<Gaps>, Blosum62 int16) (the 20,000-pair protein workload).
#include "../ref_common.h"

SEQAN_REF_UNIT(k1_m1_b0_aa16_fe0, 1, run_gaps, 1, 0, 2, 0, false, false, false, false, int16_t, AminoAcid, true)
