// Banded chain alignment (ref_banded_chain, ref_banded_chain_batch) in the benchmark library too, for
// the reference arm of bench.py's banded_chain_20k workload.
#include "../units/banded_chain.cpp"
