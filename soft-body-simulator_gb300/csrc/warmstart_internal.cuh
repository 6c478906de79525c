// Device buffers of the learned warm start (warmstart.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "xpbd_internal.cuh"

namespace sbs {

struct WarmDev {
    float* feat;          // [V][16] features
    float* delta;         // [V][3] MLP displacement guess
    float4* xpred;        // [V] predicted positions of the substep
    uint32_t* inc_start;  // [V + 1] CSR of incident tet slots
    uint32_t* inc;        // [4T]
};

cudaError_t launch_features(const SceneDev& s, const WarmDev& w, const StepParams& p, cudaStream_t st);
cudaError_t launch_fit_segment(const SceneDev& s, const WarmDev& w, const StepParams& p, uint32_t b, uint32_t e,
                               cudaStream_t st);

}  // namespace sbs
