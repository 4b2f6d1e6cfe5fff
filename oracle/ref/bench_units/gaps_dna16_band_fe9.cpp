// Reference-arm instantiation: banded globalAlignment(ExecutionPolicy<Parallel, Vectorial>,
// StringSet<Gaps>, StringSet<Gaps>, Score<int16_t, Simple>, AlignConfig<true, false, false, true>,
// lower, upper) followed by getCigarString (the read-verification workload).
#include "../ref_common.h"

SEQAN_REF_UNIT(k1_m0_b1_dna16_fe9, 1, run_gaps, 0, 1, 0, 9, true, false, false, true, int16_t, Dna5, false)
