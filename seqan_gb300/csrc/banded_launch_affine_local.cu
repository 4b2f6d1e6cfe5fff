// banded_launch_affine_local.cu -- the banded kernel's affine local instances (see banded_launch.cuh).
#include "banded_launch.cuh"

namespace gba {

BandLauncher pick_banded_affine_local(bool m, bool t) { return banded_launch::pick<true, true, false>(m, t); }

}  // namespace gba
