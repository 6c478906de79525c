// Per-vertex warm-start MLP: 16 -> 128 -> 128 -> 128 -> 3, SiLU after the
// three hidden layers.  The per-layer forward and backward passes, the
// loss, Adam on FP32 master weights, and the warp-level mma.sync GEMM
// engine (the tcgen05 engine, the default, is mlp_gemm_tc.cu); nothing
// calls a library GEMM.
//
// Layout: activations row-major [n][features], plus transposed BF16 copies
// [features][n] for the weight-gradient products; weights [out][in]
// row-major (FP32 master + BF16 copy + transposed BF16 copy); inputs are
// normalised inside the network ((x - mean) / std) and outputs scaled by
// out_scale, so callers pass raw features and receive raw displacements.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/sbs_gpu.h"
#include "mlp_internal.cuh"
#include "launch_count.cuh"

namespace sbs {

// --------------------------------------------------------------------------
// Generic BF16 GEMM on the warp-level tensor-core path (mma.sync m16n8k16),
// the comparison engine for the tcgen05 GEMM of mlp_gemm_tc.cu; both take the
// same GemmArgs (mlp_internal.cuh).  CTA tile 64 x 64, k-step 32, 4 warps of
// 32 x 32.
constexpr int GM = 64, GN = 64, GK = 32, GPAD = 8;

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

__global__ void __launch_bounds__(128) k_gemm(GemmArgs g) {
    __shared__ __align__(16) __nv_bfloat16 As[GM][GK + GPAD];
    __shared__ __align__(16) __nv_bfloat16 Bs[GN][GK + GPAD];  // n-major, k contiguous
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int gid = lane >> 2, tig = lane & 3;
    const int m0 = blockIdx.x * GM, n0 = blockIdx.y * GN;
    const int kper = g.splitk > 1 ? ((g.K + g.splitk * GK - 1) / (g.splitk * GK)) * GK : g.K;
    const int kbeg = g.splitk > 1 ? blockIdx.z * kper : 0;
    const int kend = g.splitk > 1 ? min(g.K, kbeg + kper) : g.K;
    const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
    float acc[2][4][4];
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0f;
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    for (int k0 = kbeg; k0 < kend; k0 += GK) {
        for (int e = tid; e < GM * GK; e += 128) {
            const int mm = e / GK, kk = e % GK;
            const int m = m0 + mm, k = k0 + kk;
            As[mm][kk] = (m < g.M && k < kend) ? g.A[m * g.sam + k * g.sak] : zero;
        }
        for (int e = tid; e < GN * GK; e += 128) {
            const int nn = e / GK, kk = e % GK;
            const int n = n0 + nn, k = k0 + kk;
            Bs[nn][kk] = (n < g.N && k < kend) ? g.B[k * g.sbk + n * g.sbn] : zero;
        }
        __syncthreads();
#pragma unroll
        for (int ks = 0; ks < GK; ks += 16) {
            uint32_t a[2][4], b[4][2];
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const int r = wm + i * 16 + gid;
                a[i][0] = *reinterpret_cast<const uint32_t*>(&As[r][ks + tig * 2]);
                a[i][1] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + tig * 2]);
                a[i][2] = *reinterpret_cast<const uint32_t*>(&As[r][ks + tig * 2 + 8]);
                a[i][3] = *reinterpret_cast<const uint32_t*>(&As[r + 8][ks + tig * 2 + 8]);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int c = wn + j * 8 + gid;
                b[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + tig * 2]);
                b[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[c][ks + tig * 2 + 8]);
            }
#pragma unroll
            for (int i = 0; i < 2; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], a[i], b[j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const int m = m0 + wm + i * 16 + gid + (r >= 2 ? 8 : 0);
                const int n = n0 + wn + j * 8 + tig * 2 + (r & 1);
                if (m >= g.M || n >= g.N) continue;
                float v = acc[i][j][r];
                float* cp = g.C + (long long)m * g.ldc + n;
                if (g.splitk > 1) {
                    g.ws[(size_t)blockIdx.z * g.M * g.N + (size_t)m * g.N + n] = v;
                    continue;
                }
                if (g.beta != 0.0f) v += g.beta * *cp;
                if (g.bias) v += g.bias[n];
                if (g.dsilu) v *= silu_grad(g.dsilu[(long long)m * g.ldc + n]);
                if (g.C) *cp = v;
                if (g.Cb) g.Cb[(long long)m * g.ldc + n] = __float2bfloat16(v);
                if (g.Act) g.Act[(long long)m * g.ldc + n] = __float2bfloat16(silu(v));
                if (g.T) g.T[(long long)n * g.ldt + m] = __float2bfloat16(g.Act ? silu(v) : v);
            }
}

// C[i] = sum over the K slices z = 0, 1, ... of ws[z][i] in a fixed order:
// four threads per element take consecutive quarters of the slices (each
// added in slice order), and the quarters are added in order.  Split-K
// products come out the same bit for bit on every run (an atomic
// accumulation would add the slices in whatever order they finish).
__global__ void k_splitk_sum(const float* __restrict__ ws, float* __restrict__ C, int mn, int splitk) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const int i = (int)(t >> 2), p = (int)(t & 3);
    const int per = (splitk + 3) / 4, z0 = p * per, z1 = min(splitk, z0 + per);
    float s = 0.0f;
    if (i < mn) {
#pragma unroll 8
        for (int z = z0; z < z1; ++z) s += ws[(size_t)z * mn + i];
    }
    // the four quarters, in order (lanes 4q .. 4q + 3 of a warp hold one element)
    const float s1 = __shfl_down_sync(0xffffffffu, s, 1), s2 = __shfl_down_sync(0xffffffffu, s, 2),
                s3 = __shfl_down_sync(0xffffffffu, s, 3);
    if (p == 0 && i < mn) C[i] = ((s + s1) + s2) + s3;
}

cudaError_t splitk_sum(const float* ws, float* C, int mn, int splitk, cudaStream_t st) {
    k_splitk_sum<<<(int)(((long long)mn * 4 + 255) / 256), 256, 0, st>>>(ws, C, mn, splitk);
    count_launch();
    return cudaGetLastError();
}

cudaError_t gemm_mma_sync(const GemmArgs& g, cudaStream_t st) {
    if (g.M <= 0 || g.N <= 0) return cudaSuccess;
    dim3 grid((g.M + GM - 1) / GM, (g.N + GN - 1) / GN, g.splitk > 1 ? g.splitk : 1);
    k_gemm<<<grid, 128, 0, st>>>(g);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the slices' sum into C (ldc == N for the split-K products)
    if (g.splitk > 1) return splitk_sum(g.ws, g.C, g.M * g.N, g.splitk, st);
    return cudaSuccess;
}

// the handle's engine; the tcgen05 kernel reports a timed-out wait in tc_err
static cudaError_t gemm(const MlpDev& d, GemmArgs g, cudaStream_t st) {
    g.err = d.tc_err;
    g.err_code = (int)SBS_ETIMEOUT;
    return d.engine == kGemmMmaSync ? gemm_mma_sync(g, st) : gemm_tc(g, st);
}

// split-K slices of a weight-gradient product over n rows (512 rows or more a slice)
static int splitk_for(int n) { return std::max(1, std::min(kMaxSplitK, n / 512)); }

// --------------------------------------------------------------------------
// Elementwise kernels

// xn = bf16((x - mean) / std), x [n][16]; xnT [16][n] its transpose (optional)
__global__ void k_norm_in(const float* x, const float* mean, const float* inv_std, __nv_bfloat16* xn,
                          __nv_bfloat16* xnT, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kIn) return;
    const int f = i % kIn;
    const __nv_bfloat16 v = __float2bfloat16((x[i] - mean[f]) * inv_std[f]);
    xn[i] = v;
    if (xnT) xnT[(long long)f * n + i / kIn] = v;
}

// y = z4 * out_scale (raw output), z4 [n][3]
__global__ void k_scale_out(const float* z4, const float* scale, float* y, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * kOut) return;
    y[i] = z4[i] * scale[i % kOut];
}

// loss = mean_i sum_o (z4 - t / scale)^2 ; dz4 = 2 (z4 - t/scale) / n  (bf16 and
// the transposed bf16 copy dz4T [3][n])
__global__ void k_loss(const float* z4, const float* t, const float* scale, __nv_bfloat16* dz4b,
                       __nv_bfloat16* dz4T, float* loss_acc, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e2 = 0.0f;
    if (i < n * kOut) {
        const float d = z4[i] - t[i] / scale[i % kOut];
        const __nv_bfloat16 b = __float2bfloat16(2.0f * d / (float)n);
        dz4b[i] = b;
        dz4T[(long long)(i % kOut) * n + i / kOut] = b;
        e2 = d * d;
    }
    for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    __shared__ float warp_sum[8];
    if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = e2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float b = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += warp_sum[w];
        atomicAdd(loss_acc, b / (float)n);   // the reported loss only; gradients take no atomics
    }
}

// db[o] = sum_r dzT[o][r] (the bias gradient from the transposed BF16 output
// gradient): one block per row, 16-byte loads where aligned, a fixed-order
// tree over the threads' partial sums.
__global__ void k_rowsum_bf16(const __nv_bfloat16* __restrict__ X, long long ld, int n, float* __restrict__ out) {
    const __nv_bfloat16* row = X + (long long)blockIdx.x * ld;
    float s = 0.0f;
    if ((ld & 7) == 0 && ((uintptr_t)X & 15) == 0) {
        const int n8 = n / 8;
        for (int q = threadIdx.x; q < n8; q += blockDim.x) {
            const uint4 u = __ldg(reinterpret_cast<const uint4*>(row) + q);
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float2 f = __bfloat1622float2(h[e]);
                s += f.x + f.y;
            }
        }
        for (int r = n8 * 8 + threadIdx.x; r < n; r += blockDim.x) s += __bfloat162float(row[r]);
    } else {
        for (int r = threadIdx.x; r < n; r += blockDim.x) s += __bfloat162float(row[r]);
    }
    __shared__ float sh[256];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

// Where parameter i's BF16 copy goes in the transposed weight copies: weight
// (o, c) of layer l (row-major [out][in] at woff[l]) to woff[l] + c * out + o;
// biases keep their place.
struct LayerMap {
    int woff[4], fin[4], fout[4];
};

__device__ __forceinline__ int transposed_index(const LayerMap& L, int i) {
#pragma unroll
    for (int l = 0; l < 4; ++l) {
        const int q = i - L.woff[l];
        if (q >= 0 && q < L.fin[l] * L.fout[l]) return L.woff[l] + (q % L.fin[l]) * L.fout[l] + q / L.fin[l];
    }
    return i;
}

// Adam on the FP32 masters, then refresh the BF16 copies (plain and transposed).
__global__ void k_adam(float* w, const float* gr, float* m1, float* m2, __nv_bfloat16* wb, __nv_bfloat16* wbT,
                       LayerMap L, int count, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float g = gr[i];
    const float a = b1 * m1[i] + (1.0f - b1) * g;
    const float b = b2 * m2[i] + (1.0f - b2) * g * g;
    m1[i] = a;
    m2[i] = b;
    const float v = w[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
    w[i] = v;
    wb[i] = __float2bfloat16(v);
    wbT[transposed_index(L, i)] = __float2bfloat16(v);
}

__global__ void k_to_bf16(const float* w, __nv_bfloat16* wb, __nv_bfloat16* wbT, LayerMap L, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    wb[i] = __float2bfloat16(w[i]);
    wbT[transposed_index(L, i)] = __float2bfloat16(w[i]);
}

static LayerMap layer_map(const MlpDev& d) {
    LayerMap L;
    const int fin[4] = {kIn, kHid, kHid, kHid}, fout[4] = {kHid, kHid, kHid, kOut};
    for (int l = 0; l < 4; ++l) {
        L.woff[l] = d.woff[l];
        L.fin[l] = fin[l];
        L.fout[l] = fout[l];
    }
    return L;
}

// gather rows idx[0..n) of (x, t) into contiguous batch buffers
__global__ void k_gather(const float* x, const float* t, const uint32_t* idx, float* xb, float* tb, int n) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const uint32_t s = idx[r];
    for (int f = 0; f < kIn; ++f) xb[r * kIn + f] = x[(size_t)s * kIn + f];
    for (int o = 0; o < kOut; ++o) tb[r * kOut + o] = t[(size_t)s * kOut + o];
}

// idx[r] = hash(seed, step, r) mod n_data (sampling with replacement)
__global__ void k_sample(uint32_t* idx, int n, uint32_t n_data, unsigned long long seed) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    unsigned long long z = seed + 0x9e3779b97f4a7c15ull * (unsigned long long)(r + 1);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    z ^= z >> 31;
    idx[r] = (uint32_t)(z % n_data);
}

static inline int nb(long long n, int b = 256) { return (int)((n + b - 1) / b); }

// --------------------------------------------------------------------------
// Network passes on device buffers (MlpDev holds weights and workspace).

cudaError_t mlp_forward_dev(MlpDev& d, const float* x, int n, float* y_raw, cudaStream_t st, bool keep_t) {
    cudaError_t e;
    if ((e = mlp_reserve(d, n)) != cudaSuccess) return e;
    if (keep_t && (e = mlp_reserve_train(d, n)) != cudaSuccess) return e;
    k_norm_in<<<nb((long long)n * kIn), 256, 0, st>>>(x, d.mean, d.inv_std, d.xn, keep_t ? d.xnT : nullptr, n);
    count_launch();
    const __nv_bfloat16* in = d.xn;
    int kin = kIn;
    for (int l = 0; l < 3; ++l) {
        GemmArgs g{};
        g.A = in; g.sam = kin; g.sak = 1;
        g.B = d.wb[l]; g.sbk = 1; g.sbn = kin;        // B(k, n) = W[n][k]
        g.C = d.z[l]; g.ldc = kHid; g.beta = 0.0f; g.bias = d.b[l];
        g.Act = d.a[l];
        if (keep_t) {
            g.T = d.aT[l];
            g.ldt = n;
        }
        g.M = n; g.N = kHid; g.K = kin;
        if ((e = gemm(d, g, st)) != cudaSuccess) return e;
        in = d.a[l];
        kin = kHid;
    }
    GemmArgs g{};
    g.A = d.a[2]; g.sam = kHid; g.sak = 1;
    g.B = d.wb[3]; g.sbk = 1; g.sbn = kHid;
    g.C = d.z[3]; g.ldc = kOut; g.beta = 0.0f; g.bias = d.b[3];
    g.M = n; g.N = kOut; g.K = kHid;
    if ((e = gemm(d, g, st)) != cudaSuccess) return e;
    if (y_raw) {
        k_scale_out<<<nb((long long)n * kOut), 256, 0, st>>>(d.z[3], d.out_scale, y_raw, n);
        count_launch();
    }
    return cudaGetLastError();
}

// Loss and gradient w.r.t. all parameters (into d.grad) for n rows.  Every
// product reads its operands K-contiguous: the weight gradients
// dW_l = dz_l^T act_{l-1} from the transposed copies dzT_l [out][n] and
// actT_{l-1} [in][n] that the epilogues before them wrote, the input
// gradients dz_l W_l from W_l^T; the SiLU backward is the input-gradient
// product's epilogue.
cudaError_t mlp_backward_dev(MlpDev& d, const float* x, const float* t, int n, cudaStream_t st) {
    cudaError_t e;
    if ((e = mlp_forward_dev(d, x, n, nullptr, st, true)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(d.loss, 0, sizeof(float), st)) != cudaSuccess) return e;
    k_loss<<<nb((long long)n * kOut), 256, 0, st>>>(d.z[3], t, d.out_scale, d.dzb[3], d.dzT[3], d.loss, n);
    count_launch();
    const int fin[4] = {kIn, kHid, kHid, kHid};
    const int fout[4] = {kHid, kHid, kHid, kOut};
    for (int l = 3; l >= 0; --l) {
        // dW_l[o][i] = sum_r dz_l[r][o] * act_{l-1}[r][i]
        GemmArgs g{};
        g.A = d.dzT[l]; g.sam = n; g.sak = 1;           // A(m=o, k=r) = dzT[o][r]
        g.B = l == 0 ? d.xnT : d.aT[l - 1];
        g.sbk = 1; g.sbn = n;                           // B(k=r, n=i) = actT[i][r]
        g.C = d.grad + d.woff[l]; g.ldc = fin[l]; g.beta = 0.0f;
        g.M = fout[l]; g.N = fin[l]; g.K = n;
        g.splitk = splitk_for(n);
        g.ws = d.splitk_ws;
        if ((e = gemm(d, g, st)) != cudaSuccess) return e;
        // db_l[o] = sum_r dz_l[r][o]
        k_rowsum_bf16<<<fout[l], 256, 0, st>>>(d.dzT[l], n, n, d.grad + d.boff[l]);
        count_launch();
        if (l == 0) break;
        // dz_{l-1}[r][i] = SiLU'(z_{l-1}[r][i]) sum_o dz_l[r][o] * W_l[o][i]
        GemmArgs h{};
        h.A = d.dzb[l]; h.sam = fout[l]; h.sak = 1;
        h.B = d.wbT[l]; h.sbk = 1; h.sbn = fout[l];     // B(k=o, n=i) = W^T[i][o]
        h.C = nullptr; h.ldc = kHid; h.beta = 0.0f;
        h.dsilu = d.z[l - 1];
        h.Cb = d.dzb[l - 1];
        h.T = d.dzT[l - 1]; h.ldt = n;
        h.M = n; h.N = fin[l]; h.K = fout[l];
        if ((e = gemm(d, h, st)) != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

cudaError_t mlp_adam_dev(MlpDev& d, float lr, cudaStream_t st) {
    d.step += 1;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const float c1 = 1.0f - powf(b1, (float)d.step), c2 = 1.0f - powf(b2, (float)d.step);
    k_adam<<<nb(kParams), 256, 0, st>>>(d.w, d.grad, d.m1, d.m2, d.wball, d.wballT, layer_map(d), kParams, lr, b1, b2,
                                        eps, c1, c2);
    count_launch();
    return cudaGetLastError();
}

cudaError_t mlp_sync_bf16(MlpDev& d, cudaStream_t st) {
    k_to_bf16<<<nb(kParams), 256, 0, st>>>(d.w, d.wball, d.wballT, layer_map(d), kParams);
    count_launch();
    return cudaGetLastError();
}

cudaError_t mlp_train_steps(MlpDev& d, int steps, int batch, float lr, unsigned long long seed, cudaStream_t st) {
    cudaError_t e;
    if ((e = mlp_reserve(d, batch)) != cudaSuccess) return e;
    for (int s = 0; s < steps; ++s) {
        k_sample<<<nb(batch), 256, 0, st>>>(d.idx, batch, d.n_data, seed + 1000003ull * (unsigned long long)d.step);
        count_launch();
        k_gather<<<nb(batch), 256, 0, st>>>(d.data_x, d.data_t, d.idx, d.bx, d.bt, batch);
        count_launch();
        if ((e = mlp_backward_dev(d, d.bx, d.bt, batch, st)) != cudaSuccess) return e;
        if ((e = mlp_adam_dev(d, lr, st)) != cudaSuccess) return e;
    }
    return cudaGetLastError();
}

}  // namespace sbs
