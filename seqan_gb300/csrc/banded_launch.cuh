// banded_launch.cuh -- launchers of the banded kernel's instances.  The instances are split over
// four translation units by gap model and mode (banded_launch_*.cu) so that they compile in
// parallel: the register form of the kernel is the largest code in the engine.
#pragma once

#include "dp_banded_kernels.cuh"

#include <cuda_runtime.h>

namespace gba {

using BandLauncher = void (*)(const BandArgs &, int, size_t, cudaStream_t);

// One per unit: pick_banded_<gap model><mode>(matrix, trace); the global units also hold the
// AlignExtend_ instances (pick_banded_ext_<gap model>).
BandLauncher pick_banded_affine_global(bool matrix, bool trace);
BandLauncher pick_banded_affine_local(bool matrix, bool trace);
BandLauncher pick_banded_linear_global(bool matrix, bool trace);
BandLauncher pick_banded_linear_local(bool matrix, bool trace);
BandLauncher pick_banded_ext_affine(bool matrix, bool trace);
BandLauncher pick_banded_ext_linear(bool matrix, bool trace);

namespace banded_launch {

constexpr int kLaunchBlock = 128;       // threads per block (one pair per thread)
constexpr int kMaxBandSlots = 512;      // widest band the engine accepts (band_upper - band_lower + 1)
// Bands of at most kSmallBandWidth diagonals use the 64-slot instance: bands of at most
// kBandFastW diagonals run the register form there, the others keep 64-entry slot arrays in local
// memory (the 512-entry arrays of wide bands, 6 KB per thread, overflow L1 into L2 traffic).
constexpr int kSmallBandWidth = 64;

template <bool A, bool L, bool M, bool T, bool XT>
void launch(const BandArgs &args, int grid, size_t smem, cudaStream_t s)
{
    if (args.upper - args.lower + 1 <= kSmallBandWidth)
        k_dp_banded<A, L, M, T, kSmallBandWidth, XT><<<grid, kLaunchBlock, smem, s>>>(args);
    else
        k_dp_banded<A, L, M, T, kMaxBandSlots, XT><<<grid, kLaunchBlock, smem, s>>>(args);
}

template <bool A, bool L, bool XT>
BandLauncher pick(bool m, bool t)
{
    static const BandLauncher table[4] = {launch<A, L, false, false, XT>, launch<A, L, false, true, XT>,
                                          launch<A, L, true, false, XT>, launch<A, L, true, true, XT>};
    return table[(m ? 2 : 0) | (t ? 1 : 0)];
}

}  // namespace banded_launch
}  // namespace gba
