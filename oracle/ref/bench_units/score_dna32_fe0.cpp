// Reference-arm instantiation: globalAlignmentScore(ExecutionPolicy<Parallel, Vectorial>, ...) with
// Score<int, Simple> and AlignConfig<> (the 1,024 x 150 bp linear workload).
#include "../ref_common.h"

SEQAN_REF_UNIT(k0_m0_b0_dna32_fe0, 0, run_score, 0, 0, 1, 0, false, false, false, false, int32_t, Dna5, false)
