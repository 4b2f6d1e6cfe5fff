// banded_launch_affine_global.cu -- the banded kernel's affine global instances (see banded_launch.cuh).
#include "banded_launch.cuh"

namespace gba {

BandLauncher pick_banded_affine_global(bool m, bool t) { return banded_launch::pick<true, false, false>(m, t); }

BandLauncher pick_banded_ext_affine(bool m, bool t) { return banded_launch::pick<true, false, true>(m, t); }

}  // namespace gba
