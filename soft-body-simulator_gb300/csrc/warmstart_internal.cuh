// Device buffers of the learned warm start (warmstart.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "xpbd_internal.cuh"

namespace sbs {

struct WarmDev {
    float* feat;          // [V][16] features; [3..6) is the previous substep's solve displacement
    float* delta;         // [V][3] MLP correction to that displacement
    float4* xpred;        // [V] predicted positions of the last substep that computed features
    uint32_t* inc_start;  // [V + 1] CSR of incident tet slots
    uint32_t* inc;        // [4T]
    float4* tet_f;        // [3T] deformation gradient of each tet at x_pred (rows, .w unused)
};

cudaError_t launch_features(const SceneDev& s, const WarmDev& w, const StepParams& p, int dprev_valid,
                            cudaStream_t st);
cudaError_t launch_fit_segment(const SceneDev& s, const WarmDev& w, const StepParams& p, uint32_t b, uint32_t e,
                               int first, cudaStream_t st);
cudaError_t launch_carry(const SceneDev& s, const WarmDev& w, cudaStream_t st);
cudaError_t launch_judge_fallback(const SceneDev& s, const WarmDev& w, const JudgeDev* j, cudaStream_t st);
cudaError_t launch_judge_end(JudgeDev* j, int substep, cudaStream_t st);

}  // namespace sbs
