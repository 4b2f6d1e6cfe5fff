// banded_launch_linear_global.cu -- the banded kernel's linear global instances (see banded_launch.cuh).
#include "banded_launch.cuh"

namespace gba {

BandLauncher pick_banded_linear_global(bool m, bool t) { return banded_launch::pick<false, false, false>(m, t); }

BandLauncher pick_banded_ext_linear(bool m, bool t) { return banded_launch::pick<false, false, true>(m, t); }

}  // namespace gba
