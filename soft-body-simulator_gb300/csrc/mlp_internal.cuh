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
    __nv_bfloat16* dzb[4] = {nullptr, nullptr, nullptr, nullptr};
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
    __nv_bfloat16* wballT = nullptr;   // per layer W^T [in][out] (BF16), operand of the backward da products
    const __nv_bfloat16* wbT[4];
    int engine = 0;               // GemmEngine of the training products
    // transposed BF16 copies [features][rows] (ld = rows of the batch), operands
    // of the weight-gradient products: inputs, hidden activations, output gradients
    int cap_t = 0;
    __nv_bfloat16* xnT = nullptr;
    __nv_bfloat16* aT[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16* dzT[4] = {nullptr, nullptr, nullptr, nullptr};
};

// K slices of a split-K weight-gradient product at most
constexpr int kMaxSplitK = 256;

// One BF16 GEMM with FP32 accumulation and a fused epilogue:
//   C[m, n] = beta * C[m, n] + sum_k A(m, k) * B(k, n) (+ bias[n])
// with A(m, k) = A[m * sam + k * sak] and B(k, n) = B[k * sbk + n * sbn]
// (arbitrary strides, so transposes are free).  Epilogue, in this order:
// bias; times SiLU'(dsilu[m * ldc + n]) when dsilu is set (the backward pass
// through a SiLU whose input was dsilu); the FP32 result into C; optional
// BF16 copies: Cb = the result, Act = SiLU(result); optional transposed BF16
// copy T[n * ldt + m] of Act (or of Cb when Act is null).
struct GemmArgs {
    const __nv_bfloat16* A;
    long long sam, sak;
    const __nv_bfloat16* B;
    long long sbk, sbn;
    float* C;             // [M x N] row-major, ldc
    long long ldc;
    float beta;
    const float* bias;    // [N] or null
    const float* dsilu;   // [M x N] with ldc, or null
    __nv_bfloat16* Cb;    // ld = ldc
    __nv_bfloat16* Act;   // ld = ldc
    __nv_bfloat16* T;     // [N x M], ld = ldt
    long long ldt;
    int M, N, K;
    int splitk;           // > 1: blockIdx.z takes a K slice and writes its partial product
                          // to ws[z][M x N]; k_splitk_sum then adds the slices in order
                          // (split products take no epilogue but the sum into C)
    float* ws;
    int* err;             // tcgen05 engine: set to err_code when a wait timed out
    int err_code;
};

// SiLU and its derivative with the fast exponential and division (relative
// error a few 2^-23; the results are rounded to BF16 or multiplied into BF16
// products next)
__device__ __forceinline__ float silu(float z) { return __fdividef(z, 1.0f + __expf(-z)); }
// d SiLU / dz = s (1 + z (1 - s)), s = sigmoid(z)
__device__ __forceinline__ float silu_grad(float z) {
    const float s = __fdividef(1.0f, 1.0f + __expf(-z));
    return s * (1.0f + z * (1.0f - s));
}

// GEMM engines: the tcgen05 kernel (mlp_gemm_tc.cu) and the mma.sync one (mlp.cu)
enum GemmEngine { kGemmTc = 0, kGemmMmaSync = 1 };
cudaError_t gemm_tc(const GemmArgs& g, cudaStream_t st);
cudaError_t gemm_mma_sync(const GemmArgs& g, cudaStream_t st);
cudaError_t splitk_sum(const float* ws, float* C, int mn, int splitk, cudaStream_t st);

cudaError_t mlp_reserve(MlpDev& d, int n);
// the transposed training copies for n rows as well
cudaError_t mlp_reserve_train(MlpDev& d, int n);
// per-layer forward; keep_t also writes the transposed copies the backward pass reads
cudaError_t mlp_forward_dev(MlpDev& d, const float* x, int n, float* y_raw, cudaStream_t st, bool keep_t = false);
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
