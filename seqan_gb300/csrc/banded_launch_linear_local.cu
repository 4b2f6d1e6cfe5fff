// banded_launch_linear_local.cu -- the banded kernel's linear local instances (see banded_launch.cuh).
#include "banded_launch.cuh"

namespace gba {

BandLauncher pick_banded_linear_local(bool m, bool t) { return banded_launch::pick<false, true, false>(m, t); }

}  // namespace gba
