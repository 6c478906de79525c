// C ABI of the warm-start MLP (declarations in include/sbs_gpu.h).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sbs_gpu.h"
#include "mlp_internal.cuh"

using namespace sbs;


namespace sbs {

static cudaError_t alloc_ws(void** p, size_t bytes) { return cudaMalloc(p, bytes ? bytes : 1); }

cudaError_t mlp_reserve(MlpDev& d, int n) {
    if (n <= d.cap) return cudaSuccess;
    void* ptrs[] = {d.xn, d.z[0], d.z[1], d.z[2], d.z[3], d.a[0], d.a[1], d.a[2], d.dzb[0], d.dzb[1], d.dzb[2],
                    d.dzb[3], d.idx, d.bx, d.bt};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    const size_t N = (size_t)n;
    cudaError_t e = cudaSuccess;
#define WS(ptr, bytes) \
    if (e == cudaSuccess) e = alloc_ws((void**)&(ptr), (bytes))
    WS(d.xn, N * kIn * sizeof(__nv_bfloat16));
    for (int l = 0; l < 3; ++l) {
        WS(d.z[l], N * kHid * sizeof(float));
        WS(d.a[l], N * kHid * sizeof(__nv_bfloat16));
        WS(d.dzb[l], N * kHid * sizeof(__nv_bfloat16));
    }
    WS(d.z[3], N * kOut * sizeof(float));
    WS(d.dzb[3], N * kOut * sizeof(__nv_bfloat16));
    WS(d.idx, N * sizeof(uint32_t));
    WS(d.bx, N * kIn * sizeof(float));
    WS(d.bt, N * kOut * sizeof(float));
#undef WS
    d.cap = e == cudaSuccess ? n : 0;
    return e;
}

cudaError_t mlp_reserve_train(MlpDev& d, int n) {
    if (n <= d.cap_t) return cudaSuccess;
    void* ptrs[] = {d.xnT, d.aT[0], d.aT[1], d.aT[2], d.dzT[0], d.dzT[1], d.dzT[2], d.dzT[3]};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    const size_t N = (size_t)n;
    cudaError_t e = cudaSuccess;
#define WS(ptr, bytes) \
    if (e == cudaSuccess) e = alloc_ws((void**)&(ptr), (bytes))
    WS(d.xnT, N * kIn * sizeof(__nv_bfloat16));
    for (int l = 0; l < 3; ++l) {
        WS(d.aT[l], N * kHid * sizeof(__nv_bfloat16));
        WS(d.dzT[l], N * kHid * sizeof(__nv_bfloat16));
    }
    WS(d.dzT[3], N * kOut * sizeof(__nv_bfloat16));
#undef WS
    d.cap_t = e == cudaSuccess ? n : 0;
    return e;
}

}  // namespace sbs

static sbs_status mfail(sbs_mlp* m, sbs_status s, const std::string& msg) {
    if (m) m->err = msg;
    return s;
}

#define MCU(m, call)                                                                              \
    do {                                                                                          \
        cudaError_t _e = (call);                                                                  \
        if (_e != cudaSuccess) return mfail((m), SBS_ECUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

static void free_all(sbs_mlp* m) {
    MlpDev& d = m->d;
    void* ptrs[] = {d.xn, d.z[0], d.z[1], d.z[2], d.z[3], d.a[0], d.a[1], d.a[2], d.dzb[0], d.dzb[1], d.dzb[2],
                    d.dzb[3], d.idx, d.bx, d.bt, d.data_x, d.data_t,
                    d.xnT, d.aT[0], d.aT[1], d.aT[2], d.dzT[0], d.dzT[1], d.dzT[2], d.dzT[3]};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (void* p : m->allocs) cudaFree(p);
}

// A tensor-core wait that timed out since the last check (the error flag is cleared).
static sbs_status check_tc(sbs_mlp* m) {
    int flag = 0;
    MCU(m, cudaMemcpyAsync(&flag, m->d.tc_err, sizeof(int), cudaMemcpyDeviceToHost, m->st));
    MCU(m, cudaStreamSynchronize(m->st));
    if (!flag) return SBS_OK;
    MCU(m, cudaMemsetAsync(m->d.tc_err, 0, sizeof(int), m->st));
    return mfail(m, SBS_ETIMEOUT, "tensor-core product: a wait timed out");
}

extern "C" {

uint32_t sbs_mlp_param_count(void) { return (uint32_t)kParams; }

sbs_status sbs_mlp_create(int32_t device, uint64_t seed, sbs_mlp** out) {
    if (!out) return SBS_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return SBS_ECUDA;
    if (device < 0 || device >= ndev) return SBS_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return SBS_ECUDA;
    sbs_mlp* m = new sbs_mlp();
    MlpDev& d = m->d;
    d.device = device;
    const int fin[4] = {kIn, kHid, kHid, kHid}, fout[4] = {kHid, kHid, kHid, kOut};
    int off = 0;
    for (int l = 0; l < 4; ++l) {
        d.woff[l] = off;
        off += fin[l] * fout[l];
        d.boff[l] = off;
        off += fout[l];
    }
    // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases (splitmix64 stream)
    std::vector<float> w(kParams, 0.0f);
    uint64_t z = seed ^ 0x5bd1e995ull;
    auto rnd = [&]() {
        z += 0x9e3779b97f4a7c15ull;
        uint64_t x = z;
        x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
        x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
        x ^= x >> 31;
        return (double)(x >> 11) * (1.0 / 9007199254740992.0);
    };
    for (int l = 0; l < 4; ++l) {
        const double bound = 1.0 / std::sqrt((double)fin[l]);
        for (int i = 0; i < fin[l] * fout[l]; ++i) w[d.woff[l] + i] = (float)((2.0 * rnd() - 1.0) * bound);
    }
    std::vector<float> ones(kIn, 1.0f), zeros(kIn, 0.0f), oscale(kOut, 1.0f);
    cudaError_t e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
    auto A = [&](void** p, size_t bytes) {
        if (e == cudaSuccess) e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) m->allocs.push_back(*p);
    };
    A((void**)&d.w, kParams * sizeof(float));
    A((void**)&d.grad, kParams * sizeof(float));
    A((void**)&d.splitk_ws, (size_t)kMaxSplitK * kHid * kHid * sizeof(float));
    A((void**)&d.m1, kParams * sizeof(float));
    A((void**)&d.m2, kParams * sizeof(float));
    A((void**)&d.wball, kParams * sizeof(__nv_bfloat16));
    A((void**)&d.wballT, kParams * sizeof(__nv_bfloat16));
    A((void**)&d.mean, kIn * sizeof(float));
    A((void**)&d.inv_std, kIn * sizeof(float));
    A((void**)&d.out_scale, kOut * sizeof(float));
    A((void**)&d.loss, sizeof(float));
    A((void**)&d.tc_err, sizeof(int));
    if (e == cudaSuccess) e = cudaMemset(d.tc_err, 0, sizeof(int));
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&d.n_sm, cudaDevAttrMultiProcessorCount, d.device);
    if (e == cudaSuccess) e = cudaMemcpy(d.w, w.data(), kParams * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d.m1, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(d.m2, 0, kParams * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(d.mean, zeros.data(), kIn * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d.inv_std, ones.data(), kIn * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d.out_scale, oscale.data(), kOut * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = mlp_sync_bf16(d, m->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
    if (e != cudaSuccess) {
        free_all(m);
        if (m->st) cudaStreamDestroy(m->st);
        delete m;
        return SBS_ECUDA;
    }
    for (int l = 0; l < 4; ++l) {
        d.wb[l] = d.wball + d.woff[l];
        d.wbT[l] = d.wballT + d.woff[l];
        d.b[l] = d.w + d.boff[l];
    }
    *out = m;
    return SBS_OK;
}

sbs_status sbs_mlp_destroy(sbs_mlp* m) {
    if (!m) return SBS_EINVAL;
    cudaSetDevice(m->d.device);
    if (m->st) cudaStreamSynchronize(m->st);
    free_all(m);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
    return SBS_OK;
}

const char* sbs_mlp_last_error(const sbs_mlp* m) { return m ? m->err.c_str() : ""; }

sbs_status sbs_mlp_get_params(sbs_mlp* m, float* params) {
    if (!m || !params) return SBS_EINVAL;
    MCU(m, cudaSetDevice(m->d.device));
    MCU(m, cudaMemcpyAsync(params, m->d.w, kParams * sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MCU(m, cudaStreamSynchronize(m->st));
    return SBS_OK;
}

sbs_status sbs_mlp_set_params(sbs_mlp* m, const float* params) {
    if (!m || !params) return SBS_EINVAL;
    for (int i = 0; i < kParams; ++i)
        if (!std::isfinite(params[i])) return mfail(m, SBS_EINVAL, "non-finite parameter");
    MCU(m, cudaSetDevice(m->d.device));
    MCU(m, cudaMemcpyAsync(m->d.w, params, kParams * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MCU(m, mlp_sync_bf16(m->d, m->st));
    MCU(m, cudaStreamSynchronize(m->st));
    return SBS_OK;
}

sbs_status sbs_mlp_set_normalization(sbs_mlp* m, const float* in_mean, const float* in_std, const float* out_scale) {
    if (!m || !in_mean || !in_std || !out_scale) return SBS_EINVAL;
    float inv[kIn];
    for (int f = 0; f < kIn; ++f) {
        if (!(in_std[f] > 0) || !std::isfinite(in_mean[f])) return mfail(m, SBS_EINVAL, "bad input normalisation");
        inv[f] = 1.0f / in_std[f];
    }
    for (int o = 0; o < kOut; ++o)
        if (!(out_scale[o] > 0)) return mfail(m, SBS_EINVAL, "bad output scale");
    MCU(m, cudaSetDevice(m->d.device));
    MCU(m, cudaMemcpyAsync(m->d.mean, in_mean, kIn * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MCU(m, cudaMemcpyAsync(m->d.inv_std, inv, kIn * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MCU(m, cudaMemcpyAsync(m->d.out_scale, out_scale, kOut * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MCU(m, cudaStreamSynchronize(m->st));
    return SBS_OK;
}

sbs_status sbs_mlp_forward(sbs_mlp* m, const float* x, uint32_t n, float* y) {
    return sbs_mlp_forward_path(m, x, n, y, 0);
}

sbs_status sbs_mlp_forward_path(sbs_mlp* m, const float* x, uint32_t n, float* y, int32_t path) {
    if (!m || !x || !y || n == 0 || n > (1u << 26) || (path != 0 && path != 1)) return SBS_EINVAL;
    MCU(m, cudaSetDevice(m->d.device));
    float *dx = nullptr, *dy = nullptr;
    MCU(m, cudaMalloc((void**)&dx, (size_t)n * kIn * sizeof(float)));
    cudaError_t e = cudaMalloc((void**)&dy, (size_t)n * kOut * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess)
        e = path == 0 ? mlp_infer_tc(m->d, dx, (int)n, dy, m->d.tc_err, (int)SBS_ETIMEOUT, m->d.n_sm, m->st)
                      : mlp_forward_dev(m->d, dx, (int)n, dy, m->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(y, dy, (size_t)n * kOut * sizeof(float), cudaMemcpyDeviceToHost, m->st);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, m->d.tc_err, sizeof(int), cudaMemcpyDeviceToHost, m->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
    cudaFree(dx);
    if (dy) cudaFree(dy);
    if (e != cudaSuccess) return mfail(m, SBS_ECUDA, cudaGetErrorString(e));
    if (flag) {
        cudaMemsetAsync(m->d.tc_err, 0, sizeof(int), m->st);
        return mfail(m, SBS_ETIMEOUT, "tensor-core inference: a wait timed out");
    }
    return SBS_OK;
}

sbs_status sbs_mlp_forward_device(sbs_mlp* m, const float* x, uint32_t n, float* y, int32_t path, float* ms) {
    if (!m || !x || !y || n == 0 || n > (1u << 26) || (path != 0 && path != 1)) return SBS_EINVAL;
    MCU(m, cudaSetDevice(m->d.device));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (ms) {
        MCU(m, cudaEventCreate(&e0));
        MCU(m, cudaEventCreate(&e1));
        MCU(m, cudaEventRecord(e0, m->st));
    }
    cudaError_t e = path == 0 ? mlp_infer_tc(m->d, x, (int)n, y, m->d.tc_err, (int)SBS_ETIMEOUT, m->d.n_sm, m->st)
                              : mlp_forward_dev(m->d, x, (int)n, y, m->st);
    if (e == cudaSuccess && ms) e = cudaEventRecord(e1, m->st);
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, m->d.tc_err, sizeof(int), cudaMemcpyDeviceToHost, m->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
    if (e == cudaSuccess && ms) e = cudaEventElapsedTime(ms, e0, e1);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (e != cudaSuccess) return mfail(m, SBS_ECUDA, cudaGetErrorString(e));
    if (flag) {
        cudaMemsetAsync(m->d.tc_err, 0, sizeof(int), m->st);
        return mfail(m, SBS_ETIMEOUT, "tensor-core inference: a wait timed out");
    }
    return SBS_OK;
}

// Mean squared error of the normalised outputs and its gradient w.r.t. all
// parameters (same layout as sbs_mlp_get_params) for n rows (host buffers).
sbs_status sbs_mlp_loss_grad(sbs_mlp* m, const float* x, const float* t, uint32_t n, float* loss, float* grad) {
    if (!m || !x || !t || n == 0 || n > (1u << 26)) return SBS_EINVAL;
    MCU(m, cudaSetDevice(m->d.device));
    float *dx = nullptr, *dt = nullptr;
    MCU(m, cudaMalloc((void**)&dx, (size_t)n * kIn * sizeof(float)));
    cudaError_t e = cudaMalloc((void**)&dt, (size_t)n * kOut * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dt, t, (size_t)n * kOut * sizeof(float), cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess) e = mlp_backward_dev(m->d, dx, dt, (int)n, m->st);
    if (e == cudaSuccess && loss) e = cudaMemcpyAsync(loss, m->d.loss, sizeof(float), cudaMemcpyDeviceToHost, m->st);
    if (e == cudaSuccess && grad)
        e = cudaMemcpyAsync(grad, m->d.grad, kParams * sizeof(float), cudaMemcpyDeviceToHost, m->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
    cudaFree(dx);
    if (dt) cudaFree(dt);
    if (e != cudaSuccess) return mfail(m, SBS_ECUDA, cudaGetErrorString(e));
    return check_tc(m);
}

sbs_status sbs_mlp_set_dataset(sbs_mlp* m, const float* x, const float* t, uint32_t n) {
    if (!m || !x || !t || n == 0) return SBS_EINVAL;
    MCU(m, cudaSetDevice(m->d.device));
    MlpDev& d = m->d;
    if (d.data_x) cudaFree(d.data_x);
    if (d.data_t) cudaFree(d.data_t);
    d.data_x = d.data_t = nullptr;
    d.n_data = 0;
    MCU(m, cudaMalloc((void**)&d.data_x, (size_t)n * kIn * sizeof(float)));
    MCU(m, cudaMalloc((void**)&d.data_t, (size_t)n * kOut * sizeof(float)));
    MCU(m, cudaMemcpyAsync(d.data_x, x, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MCU(m, cudaMemcpyAsync(d.data_t, t, (size_t)n * kOut * sizeof(float), cudaMemcpyHostToDevice, m->st));
    MCU(m, cudaStreamSynchronize(m->st));
    d.n_data = n;
    return SBS_OK;
}

// Adam steps on random batches (with replacement) of the uploaded dataset.
sbs_status sbs_mlp_train(sbs_mlp* m, uint32_t steps, uint32_t batch, float lr, uint64_t seed, float* loss) {
    if (!m || batch == 0 || batch > (1u << 22) || !(lr > 0)) return SBS_EINVAL;
    if (m->d.n_data == 0) return mfail(m, SBS_ESTATE, "no dataset");
    MCU(m, cudaSetDevice(m->d.device));
    MCU(m, mlp_train_steps(m->d, (int)steps, (int)batch, lr, seed, m->st));
    if (loss) MCU(m, cudaMemcpyAsync(loss, m->d.loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MCU(m, cudaStreamSynchronize(m->st));
    return check_tc(m);
}

sbs_status sbs_mlp_set_gemm(sbs_mlp* m, int32_t engine) {
    if (!m || (engine != kGemmTc && engine != kGemmMmaSync)) return SBS_EINVAL;
    m->d.engine = engine;
    return SBS_OK;
}

}  // extern "C"
