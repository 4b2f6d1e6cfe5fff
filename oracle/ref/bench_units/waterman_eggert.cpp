// The Waterman-Eggert enumeration (ref_local_enumerate) in the benchmark library too, for the
// reference arm of bench.py's waterman_eggert_10k workload.
#include "../units/waterman_eggert.cpp"
