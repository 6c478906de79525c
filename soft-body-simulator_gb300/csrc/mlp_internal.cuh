// Device state of the warm-start MLP (mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace sbs {

constexpr int kIn = 16, kHid = 128, kOut = 3;
constexpr int kParams = kHid * kIn + kHid + 2 * (kHid * kHid + kHid) + kOut * kHid + kOut;  // 35,587

struct MlpDev {
    int device = 0;
    // parameters: W1 b1 W2 b2 W3 b3 W4 b4 (FP32 masters), BF16 copy, Adam moments
    float* w = nullptr;
    float* grad = nullptr;
    float* m1 = nullptr;
    float* m2 = nullptr;
    __nv_bfloat16* wball = nullptr;
    int woff[4], boff[4];
    const __nv_bfloat16* wb[4];
    const float* b[4];
    long long step = 0;
    // normalisation
    float* mean = nullptr;
    float* inv_std = nullptr;
    float* out_scale = nullptr;
    // workspace for `cap` rows
    int cap = 0;
    __nv_bfloat16* xn = nullptr;
    float* z[4] = {nullptr, nullptr, nullptr, nullptr};
    __nv_bfloat16* a[3] = {nullptr, nullptr, nullptr};
    float* dz[4] = {nullptr, nullptr, nullptr, nullptr};
    __nv_bfloat16* dzb[4] = {nullptr, nullptr, nullptr, nullptr};
    float* da = nullptr;
    float* loss = nullptr;
    uint32_t* idx = nullptr;
    float* bx = nullptr;
    float* bt = nullptr;
    // training set
    float* data_x = nullptr;
    float* data_t = nullptr;
    uint32_t n_data = 0;
    int* tc_err = nullptr;     // error flag of the fused inference kernel
    int n_sm = 0;
    float* splitk_ws = nullptr;   // [kMaxSplitK][kHid x kHid] partial weight gradients
};

// K slices of a split-K weight-gradient product at most
constexpr int kMaxSplitK = 256;

cudaError_t mlp_reserve(MlpDev& d, int n);
cudaError_t mlp_forward_dev(MlpDev& d, const float* x, int n, float* y_raw, cudaStream_t st);
// Inference only (no activations kept): the fused tcgen05 kernel of
// mlp_tc.cu.  A wait that times out stores err_code into *err (if 0).
// Sets the tcgen05 inference kernel's shared-memory limit on the current device.
cudaError_t mlp_tc_configure();
cudaError_t mlp_infer_tc(const MlpDev& d, const float* x, int n, float* y, int* err, int err_code, int n_sm,
                         cudaStream_t st);
cudaError_t mlp_backward_dev(MlpDev& d, const float* x, const float* t, int n, cudaStream_t st);
cudaError_t mlp_adam_dev(MlpDev& d, float lr, cudaStream_t st);
cudaError_t mlp_sync_bf16(MlpDev& d, cudaStream_t st);
cudaError_t mlp_train_steps(MlpDev& d, int steps, int batch, float lr, unsigned long long seed, cudaStream_t st);

}  // namespace sbs

// Handle behind the C ABI's sbs_mlp.
struct sbs_mlp {
    sbs::MlpDev d;
    cudaStream_t st = nullptr;
    std::vector<void*> allocs;
    std::string err;
};
