// Host-side launch descriptor shared by the ABI layer and the step kernels.
#pragma once

#include <cuda_runtime.h>

#include "../../include/islbm.h"
#include "step_common.cuh"

namespace islbm {

struct StepLaunch {
    int precision;             // islbm_precision
    const void *fo;            // 19*N populations, storage type
    void *fn;
    const void *tables;        // Tables<C> on the host (passed by value to the kernel)
    StepConst k;
    Ctrl *ctrl;                // device
    unsigned long long n;      // 1-based number of the step being computed
    bool les, macros_on, mass;
    void *macros[4];           // rho, u, v, w (compute type) when macros_on
    const void *tiled;         // TiledConst for the tiled kernel
    const void *pmaps;         // paired kernel: the 4 tensor maps (CUtensorMap) of buffer fo, or null
    cudaStream_t stream;
};

cudaError_t launch_step_gather(const StepLaunch &L);
cudaError_t launch_step_tiled(const StepLaunch &L);
bool tiled_supported(const StepConst &k, int precision);

}  // namespace islbm
