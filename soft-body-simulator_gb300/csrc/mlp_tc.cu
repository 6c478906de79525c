// Fused inference of the warm-start MLP (16 -> 128 -> 128 -> 128 -> 3, SiLU)
// on the 5th-generation tensor cores of sm_100-class GPUs.
//
// One CTA of four tile slots per SM; each slot (two warps per TMEM lane
// quarter: 256 threads, two per tile row, each with half of the columns)
// takes 128-row tiles (rows = vertices) on its own, so one slot's epilogue
// overlaps another's MMAs.  The four weight matrices stay in shared memory
// for the CTA's lifetime (shared by the slots; staged 16 bytes at a time, the
// hidden layers' halved), in the canonical K-major layout without swizzle that
// tcgen05.mma reads through shared-memory descriptors (tc_common.cuh).  Per
// layer one elected thread issues K / 16 MMAs (M = 128, N = 128 - or 16 for
// the 3-wide output, zero-padded - K = 16 each, BF16 inputs, FP32
// accumulators in tensor memory), commits them to an mbarrier, and the slot's
// eight warps read the accumulators back with tcgen05.ld (warp w reads TMEM lanes
// 32 (w % 4).. = rows of the tile, 32 columns per load), add the bias (from
// shared memory), apply SiLU, round to BF16 pairs and write the next layer's
// A operand.  Waits on the mbarrier are bounded in time; on expiry the kernel
// records an error, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "launch_count.cuh"
#include "mlp_internal.cuh"
#include "tc_common.cuh"

namespace sbs {

namespace {

using namespace tc;

constexpr int kTileRows = 128;                    // UMMA M
constexpr int kOutPad = 16;                       // layer-4 N, padded
constexpr int kGroups = 4;                        // tile slots (thread groups) per CTA
constexpr int kSplit = 2;                         // threads per tile row: the columns are split between them
constexpr int kGroupThreads = 128 * kSplit;       // a tile slot's threads
constexpr uint32_t kTmemCols = 128;               // accumulator columns per warpgroup
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s
// shared memory carve-up (bytes, 1024-aligned pieces)
constexpr uint32_t kW1 = 0;                                   // 128 x 16
constexpr uint32_t kW2 = kW1 + kHid * kIn * 2;                // 128 x 128
constexpr uint32_t kW3 = kW2 + kHid * kHid * 2;               // 128 x 128
constexpr uint32_t kW4 = kW3 + kHid * kHid * 2;               // 16 x 128
constexpr uint32_t kGroupBase = kW4 + kOutPad * kHid * 2;     // per-warpgroup operands from here
constexpr uint32_t kA1 = 0;                                   // 128 x 16 (offset in a group's block)
constexpr uint32_t kAct = kA1 + kTileRows * kIn * 2;          // 128 x 128
constexpr uint32_t kGroupBytes = kAct + kTileRows * kHid * 2; // 36,864
constexpr uint32_t kSmemBytes = kGroupBase + kGroups * kGroupBytes;  // 221,184

struct TcArgs {
    const float* x;            // [n][16] raw features
    int x_aligned;             // x is 16-byte aligned: rows load as float4
    int n;
    const float* mean;         // [16]
    const float* inv_std;      // [16]
    const __nv_bfloat16* w[4]; // row-major [out][in]
    int w_aligned;             // all four are 16-byte aligned: rows load 8 weights at a time
    const float* b[4];
    const float* out_scale;    // [3]
    float* y;                  // [n][3]
    int* err;                  // set to err_code on a wait that timed out
    int err_code;
};

// SiLU(z) = z sigmoid(z) = (z / 2)(1 + tanh(z / 2)).  The hidden layers'
// weights and biases are halved when they are staged (a power of two, exact
// in BF16 and FP32), so the accumulator plus bias is already h = z / 2 and
// SiLU(z) = h + h tanh(h): one add, the hardware tanh approximation
// (tanh.approx.f32, relative error about 2^-11) and one FMA per element,
// before the result is rounded to BF16 (2^-8).  (The same on BF16 pairs,
// tanh.approx.bf16x2 and a pair FMA, measured no faster.)
__device__ __forceinline__ float silu_half(float h) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(h));
    return fmaf(h, t, h);
}

__device__ __forceinline__ void group_sync(uint32_t g) {
    asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(kGroupThreads) : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&p);
}

// accumulators + halved bias -> SiLU -> BF16 into the next layer's A
// operand: this thread's row, columns [c_begin, c_begin + kHid / kSplit)
__device__ __forceinline__ void hidden_epilogue(uint32_t tmem_row, const float* half_bias, uint8_t* act, int c_begin) {
    const uint32_t r = threadIdx.x & 127u;
#pragma unroll 1
    for (int c0 = c_begin; c0 < c_begin + kHid / kSplit; c0 += 32) {
        uint32_t u[32];
        tmem_ld32_async(tmem_row + (uint32_t)c0, u);
        tmem_wait_ld();
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            const float4 b0 = *reinterpret_cast<const float4*>(half_bias + c0 + g * 8);
            const float4 b1 = *reinterpret_cast<const float4*>(half_bias + c0 + g * 8 + 4);
            const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
            float y[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) y[j] = silu_half(__uint_as_float(u[g * 8 + j]) + bb[j]);
            const uint4 q = make_uint4(pack_bf16(y[0], y[1]), pack_bf16(y[2], y[3]), pack_bf16(y[4], y[5]),
                                       pack_bf16(y[6], y[7]));
            *reinterpret_cast<uint4*>(act + canon(r, (uint32_t)(c0 + g * 8), kHid)) = q;
        }
    }
}

// W [valid rows][K] (row-major BF16) -> a rows x K canonical K-major operand
// at dst, rows past `valid` zero, halved if asked (exact: a power of two)
__device__ __forceinline__ void stage_weights(uint8_t* dst, const __nv_bfloat16* __restrict__ w, int rows, int K,
                                              int valid, bool half, bool aligned) {
    const int per_row = K / 8;
    for (int i = (int)threadIdx.x; i < rows * per_row; i += (int)blockDim.x) {
        const int r = i / per_row, q = i % per_row;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (r < valid) {
            if (aligned) {
                v = __ldg(reinterpret_cast<const uint4*>(w + (size_t)r * K) + q);
            } else {
                uint32_t u[4];
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    u[e] = (uint32_t)__bfloat16_as_ushort(w[(size_t)r * K + 8 * q + 2 * e]) |
                           ((uint32_t)__bfloat16_as_ushort(w[(size_t)r * K + 8 * q + 2 * e + 1]) << 16);
                v = make_uint4(u[0], u[1], u[2], u[3]);
            }
            if (half) {
                __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&v);
                const __nv_bfloat162 c = __floats2bfloat162_rn(0.5f, 0.5f);
#pragma unroll
                for (int e = 0; e < 4; ++e) h[e] = __hmul2(h[e], c);
            }
        }
        *reinterpret_cast<uint4*>(dst + canon((uint32_t)r, (uint32_t)(8 * q), (uint32_t)K)) = v;
    }
}

__global__ void __launch_bounds__(kGroupThreads * kGroups, 1) k_mlp_infer_tc(TcArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ __align__(8) uint64_t mbar[kGroups];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail[kGroups];
    __shared__ __align__(16) float s_hbias[3][kHid];   // halved hidden-layer biases
    __shared__ __align__(16) float s_mean[kIn], s_istd[kIn];
    __shared__ float s_b4[kOut], s_scale[kOut];
    // slot g's threads: row r of its tiles, column part `part`; warp w reads
    // TMEM lanes 32 (w % 4).. = rows r of that quarter
    const uint32_t tid = threadIdx.x, warp = tid >> 5, g = tid / kGroupThreads, r = tid & 127u;
    const uint32_t part = (tid % kGroupThreads) >> 7;
    const bool leader = (tid % kGroupThreads) == 0;

    // weights -> canonical layouts (hidden layers halved, W4 zero-padded to
    // 16 rows), biases and normalisation -> shared memory, all warpgroups;
    // eight consecutive k of a row (16 bytes) are one row of a core matrix
    stage_weights(sm + kW1, a.w[0], kHid, kIn, kHid, true, a.w_aligned);
    stage_weights(sm + kW2, a.w[1], kHid, kHid, kHid, true, a.w_aligned);
    stage_weights(sm + kW3, a.w[2], kHid, kHid, kHid, true, a.w_aligned);
    stage_weights(sm + kW4, a.w[3], kOutPad, kHid, kOut, false, a.w_aligned);
    for (uint32_t i = tid; i < 3u * kHid; i += blockDim.x) s_hbias[i / kHid][i % kHid] = 0.5f * a.b[i / kHid][i % kHid];
    if (tid < (uint32_t)kIn) {
        s_mean[tid] = a.mean[tid];
        s_istd[tid] = a.inv_std[tid];
    }
    if (tid < (uint32_t)kOut) {
        s_b4[tid] = a.b[3][tid];
        s_scale[tid] = a.out_scale[tid];
    }
    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), kTmemCols * kGroups);
    if (leader) {
        s_fail[g] = 0;
        mbar_init(smem_u32(&mbar[g]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    // this warpgroup's accumulator columns; warp w of a warpgroup reads TMEM lanes 32 (w % 4)...
    const uint32_t tmem = tmem_slot + g * kTmemCols;
    const uint32_t tmem_row = tmem + (((warp & 3u) * 32u) << 16);
    const uint32_t mb = smem_u32(&mbar[g]);
    const uint32_t base = smem_u32(sm);
    uint8_t* gsm = sm + kGroupBase + g * kGroupBytes;
    const uint32_t gbase = base + kGroupBase + g * kGroupBytes;
    uint32_t parity = 0;
    const int tiles = (a.n + kTileRows - 1) / kTileRows;

    // slot g of CTA b takes tiles b + g * grid, then every grid * kGroups-th:
    // with fewer tiles than slots the tiles spread over the SMs, one slot each
    for (int tile = blockIdx.x + (int)g * gridDim.x; tile < tiles; tile += gridDim.x * kGroups) {
        const int row = tile * kTileRows + (int)r;
        const bool valid = row < a.n;
        // layer-1 A operand: normalised features (this thread's 16 / kSplit of the row)
        {
            constexpr int kPer = kIn / kSplit;
            const int k0 = (int)part * kPer;
            float xv[kPer];
            if (valid && a.x_aligned) {
                const float4* xr = reinterpret_cast<const float4*>(a.x + (size_t)row * kIn + k0);
#pragma unroll
                for (int q = 0; q < kPer / 4; ++q) {
                    const float4 f = __ldg(xr + q);
                    xv[4 * q] = f.x; xv[4 * q + 1] = f.y; xv[4 * q + 2] = f.z; xv[4 * q + 3] = f.w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < kPer; ++k) xv[k] = valid ? __ldg(&a.x[(size_t)row * kIn + k0 + k]) : 0.0f;
            }
            uint32_t h[kPer / 2];
#pragma unroll
            for (int k = 0; k < kPer; k += 2) {
                const float f0 = valid ? (xv[k] - s_mean[k0 + k]) * s_istd[k0 + k] : 0.0f;
                const float f1 = valid ? (xv[k + 1] - s_mean[k0 + k + 1]) * s_istd[k0 + k + 1] : 0.0f;
                h[k / 2] = pack_bf16(f0, f1);
            }
#pragma unroll
            for (int q = 0; q < kPer / 8; ++q)
                *reinterpret_cast<uint4*>(gsm + kA1 + canon(r, (uint32_t)(k0 + 8 * q), kIn)) =
                    make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
        }
        for (int layer = 0; layer < 4; ++layer) {
            const uint32_t K = layer == 0 ? kIn : kHid;
            const uint32_t aop = gbase + (layer == 0 ? kA1 : kAct);
            const uint32_t bop = base + (layer == 0 ? kW1 : layer == 1 ? kW2 : layer == 2 ? kW3 : kW4);
            const uint32_t idesc = instr_desc(kTileRows, layer == 3 ? kOutPad : kHid);
            fence_async_smem();
            fence_before();
            group_sync(g);
            if (leader) {
                fence_after();
                for (uint32_t s = 0; s < K / 16; ++s)
                    mma(tmem, smem_desc(aop + 256 * s, K), smem_desc(bop + 256 * s, K), idesc, s > 0 ? 1u : 0u);
                commit(mb);
            }
            const bool ok = wait_phase(mb, parity, kWaitLimitNs);
            parity ^= 1u;
            if (!ok) s_fail[g] = 1;
            group_sync(g);
            if (s_fail[g]) break;
            fence_after();
            if (layer < 3) {
                hidden_epilogue(tmem_row, s_hbias[layer], gsm + kAct, (int)part * (kHid / kSplit));
            } else if (part == 0) {
                float v[16];
                tmem_ld16(tmem_row, v);
                if (valid)
                    for (int j = 0; j < kOut; ++j) a.y[(size_t)row * kOut + j] = (v[j] + s_b4[j]) * s_scale[j];
            }
        }
        if (s_fail[g]) break;
    }
    if (s_fail[g] && leader) atomicCAS(a.err, 0, a.err_code);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        tmem_dealloc(tmem_slot, kTmemCols * kGroups);
    }
}

}  // namespace

cudaError_t mlp_tc_configure() {
    return cudaFuncSetAttribute(k_mlp_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemBytes);
}

cudaError_t mlp_infer_tc(const MlpDev& d, const float* x, int n, float* y, int* err, int err_code, int n_sm,
                         cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    // per device and cheap: set on every call (the caller may switch
    // devices), except while the stream is being captured into a graph (the
    // warm-start path sets it when the network is attached)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    if (cs == cudaStreamCaptureStatusNone && (e = mlp_tc_configure()) != cudaSuccess) return e;
    TcArgs a;
    a.x = x;
    a.x_aligned = ((uintptr_t)x & 15u) == 0;
    a.n = n;
    a.mean = d.mean;
    a.inv_std = d.inv_std;
    a.w_aligned = 1;
    for (int l = 0; l < 4; ++l) {
        a.w[l] = d.wb[l];
        a.b[l] = d.b[l];
        if ((uintptr_t)d.wb[l] & 15u) a.w_aligned = 0;
    }
    a.out_scale = d.out_scale;
    a.y = y;
    a.err = err;
    a.err_code = err_code;
    const int tiles = (n + kTileRows - 1) / kTileRows;
    // one CTA (4 tile slots of 256 threads, 216 KB) per SM; a small call
    // (fewer tiles than SMs) takes one CTA per tile rather than packing its
    // tiles into the slots of a few SMs
    const int grid = tiles < n_sm ? tiles : n_sm;
    k_mlp_infer_tc<<<grid, kGroupThreads * kGroups, kSmemBytes, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace sbs
