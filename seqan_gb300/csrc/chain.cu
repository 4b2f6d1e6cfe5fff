// chain.cu -- the banded chain alignment kernels (chain_kernels.cuh) in a translation unit of
// their own, with their launchers; gba_banded_chain (chain_host.cuh, in engine.cu) calls these.
#include <cuda_runtime.h>

#define SEQAN_GB300_CHAIN_KERNELS
#include "chain_kernels.cuh"

void launch_banded_chain(const ChainArgs &a, cudaStream_t st)
{
    k_banded_chain<<<unsigned((a.num_chains * 32 + 127) / 128), 128, 0, st>>>(a);   // one warp per chain
}

void launch_chain_pack(const chain::ChainDesc *chains, int64_t num_chains, const uint8_t *arena, int32_t max_traces,
                       const int32_t *seg_count, const int64_t *dense_off, chain::Seg *dense, cudaStream_t st)
{
    k_chain_pack<<<unsigned((num_chains + 127) / 128), 128, 0, st>>>(chains, num_chains, arena, max_traces, seg_count,
                                                                      dense_off, dense);
}
