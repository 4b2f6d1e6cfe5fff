// Reference-arm instantiation: globalAlignmentScore(ExecutionPolicy<Parallel, Vectorial>, ...) with
// Score<int16_t, Simple> and AlignConfig<> (the 100,000-pair affine DNA workload).
#include "../ref_common.h"

SEQAN_REF_UNIT(k0_m0_b0_dna16_fe0, 0, run_score, 0, 0, 0, 0, false, false, false, false, int16_t, Dna5, false)
