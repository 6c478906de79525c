// Fused inference of the warm-start MLP (16 -> 128 -> 128 -> 128 -> 3, SiLU)
// on the 5th-generation tensor cores of sm_100-class GPUs.
//
// One CTA of four warpgroups per SM; each warpgroup takes 128-row tiles
// (rows = vertices) on its own, so one warpgroup's epilogue overlaps another's
// MMAs.  The four weight matrices stay in shared memory for the CTA's
// lifetime (shared by the warpgroups), in the
// canonical K-major layout without swizzle that tcgen05.mma reads through
// shared-memory descriptors: core matrices of 8 rows x 16 bytes, element
// (r, k) at (r / 8) * SBO + (k / 8) * LBO + (r % 8) * 16 + (k % 8) * 2 with
// LBO = 128 B and SBO = (K / 8) * 128 B.  Per layer one elected thread issues
// K / 16 MMAs (M = 128, N = 128 - or 16 for the 3-wide output, zero-padded -
// K = 16 each, BF16 inputs, FP32 accumulators in tensor memory), commits
// them to an mbarrier, and the four warps read the accumulators back with
// tcgen05.ld (warp w owns TMEM lanes 32w..32w+31 = rows of the tile), add the
// bias, apply SiLU, round to BF16 and write the next layer's A operand.
// Waits on the mbarrier are bounded in time; on expiry the kernel records an
// error, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "launch_count.cuh"
#include "mlp_internal.cuh"

namespace sbs {

namespace {

constexpr int kTileRows = 128;                    // UMMA M
constexpr int kOutPad = 16;                       // layer-4 N, padded
constexpr int kGroups = 4;                        // warpgroups per CTA
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
    const float* b[4];
    const float* out_scale;    // [3]
    float* y;                  // [n][3]
    int* err;                  // set to err_code on a wait that timed out
    int err_code;
};

__device__ __forceinline__ uint32_t canon(uint32_t r, uint32_t k, uint32_t K) {
    return (r >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t K) {
    const uint64_t lbo = 128, sbo = (uint64_t)(K / 8) * 128;
    return (uint64_t)((addr & 0x3FFFF) >> 4) | ((lbo >> 4) << 16) | ((sbo >> 4) << 32) | (1ull << 46);
}

__host__ __device__ constexpr uint32_t instr_desc(uint32_t N) {
    // D f32 (bits 4-5 = 1), A bf16 (7-9 = 1), B bf16 (10-12 = 1), both
    // K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((uint32_t)(kTileRows >> 4) << 24);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(accum)
        : "memory");
}

__device__ __forceinline__ void commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

// bounded wait for the mbarrier phase `parity` to complete
__device__ __forceinline__ bool wait_phase(uint32_t mbar, uint32_t parity) {
    const unsigned long long t0 = now_ns();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mbar), "r"(parity)
            : "memory");
        if (done) return true;
        if (now_ns() - t0 > kWaitLimitNs) return false;
    }
}

__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 32 consecutive accumulator columns of this thread's row
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// SiLU as z * sigmoid(z) = z (1 + tanh(z / 2)) / 2 with the hardware tanh
// approximation (tanh.approx.f32, relative error about 2^-11); the result is
// rounded to BF16 (2^-8) next
__device__ __forceinline__ float silu_f(float z) {
    float t;
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(0.5f * z));
    return 0.5f * z * (1.0f + t);
}

__device__ __forceinline__ void group_sync(uint32_t g) {
    asm volatile("bar.sync %0, %1;" ::"r"(g + 1), "r"(128) : "memory");
}

// accumulators + bias -> SiLU -> BF16 into the next layer's A operand
__device__ __forceinline__ void hidden_epilogue(uint32_t tmem_row, const float* bias, uint8_t* act) {
    const uint32_t r = threadIdx.x & 127u;
#pragma unroll 1
    for (int c0 = 0; c0 < kHid; c0 += 32) {
        float v[32];
        tmem_ld32(tmem_row + (uint32_t)c0, v);
#pragma unroll
        for (int g = 0; g < 4; ++g) {
            __align__(16) __nv_bfloat16 h[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) h[j] = __float2bfloat16(silu_f(v[g * 8 + j] + __ldg(&bias[c0 + g * 8 + j])));
            *reinterpret_cast<uint4*>(act + canon(r, (uint32_t)(c0 + g * 8), kHid)) =
                *reinterpret_cast<const uint4*>(h);
        }
    }
}

__global__ void __launch_bounds__(128 * kGroups, 1) k_mlp_infer_tc(TcArgs a) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ __align__(8) uint64_t mbar[kGroups];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_fail[kGroups];
    const uint32_t tid = threadIdx.x, warp = tid >> 5, g = tid >> 7, r = tid & 127u;

    // weights -> canonical layouts (W4 zero-padded to 16 rows), all warpgroups
    for (uint32_t i = tid; i < (uint32_t)(kHid * kIn); i += blockDim.x) {
        const uint32_t rr = i / kIn, k = i % kIn;
        *reinterpret_cast<__nv_bfloat16*>(sm + kW1 + canon(rr, k, kIn)) = a.w[0][i];
    }
    for (uint32_t i = tid; i < (uint32_t)(kHid * kHid); i += blockDim.x) {
        const uint32_t rr = i / kHid, k = i % kHid;
        *reinterpret_cast<__nv_bfloat16*>(sm + kW2 + canon(rr, k, kHid)) = a.w[1][i];
        *reinterpret_cast<__nv_bfloat16*>(sm + kW3 + canon(rr, k, kHid)) = a.w[2][i];
    }
    for (uint32_t i = tid; i < (uint32_t)(kOutPad * kHid); i += blockDim.x) {
        const uint32_t rr = i / kHid, k = i % kHid;
        *reinterpret_cast<__nv_bfloat16*>(sm + kW4 + canon(rr, k, kHid)) =
            rr < (uint32_t)kOut ? a.w[3][rr * kHid + k] : __float2bfloat16(0.0f);
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kTmemCols * kGroups)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (r == 0) {
        s_fail[g] = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[g])) : "memory");
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

    for (int tile = blockIdx.x * kGroups + (int)g; tile < tiles; tile += gridDim.x * kGroups) {
        const int row = tile * kTileRows + (int)r;
        const bool valid = row < a.n;
        // layer-1 A operand: normalised features
        {
            __align__(16) __nv_bfloat16 h[16];
            float xv[kIn];
            if (valid && a.x_aligned) {
                // the row's 64 bytes as four 16-byte loads
                const float4* xr = reinterpret_cast<const float4*>(a.x + (size_t)row * kIn);
#pragma unroll
                for (int q = 0; q < kIn / 4; ++q) {
                    const float4 f = __ldg(xr + q);
                    xv[4 * q] = f.x; xv[4 * q + 1] = f.y; xv[4 * q + 2] = f.z; xv[4 * q + 3] = f.w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < kIn; ++k) xv[k] = valid ? __ldg(&a.x[(size_t)row * kIn + k]) : 0.0f;
            }
#pragma unroll
            for (int k = 0; k < kIn; ++k) {
                const float f = valid ? (xv[k] - __ldg(&a.mean[k])) * __ldg(&a.inv_std[k]) : 0.0f;
                h[k] = __float2bfloat16(f);
            }
            *reinterpret_cast<uint4*>(gsm + kA1 + canon(r, 0, kIn)) = *reinterpret_cast<const uint4*>(&h[0]);
            *reinterpret_cast<uint4*>(gsm + kA1 + canon(r, 8, kIn)) = *reinterpret_cast<const uint4*>(&h[8]);
        }
        for (int layer = 0; layer < 4; ++layer) {
            const uint32_t K = layer == 0 ? kIn : kHid;
            const uint32_t aop = gbase + (layer == 0 ? kA1 : kAct);
            const uint32_t bop = base + (layer == 0 ? kW1 : layer == 1 ? kW2 : layer == 2 ? kW3 : kW4);
            const uint32_t idesc = instr_desc(layer == 3 ? kOutPad : kHid);
            fence_async_smem();
            fence_before();
            group_sync(g);
            if (r == 0) {
                fence_after();
                for (uint32_t s = 0; s < K / 16; ++s)
                    mma(tmem, smem_desc(aop + 256 * s, K), smem_desc(bop + 256 * s, K), idesc, s > 0 ? 1u : 0u);
                commit(mb);
            }
            const bool ok = wait_phase(mb, parity);
            parity ^= 1u;
            if (!ok) s_fail[g] = 1;
            group_sync(g);
            if (s_fail[g]) break;
            fence_after();
            if (layer < 3) {
                hidden_epilogue(tmem_row, a.b[layer], gsm + kAct);
            } else {
                float v[16];
                tmem_ld16(tmem_row, v);
                if (valid)
                    for (int j = 0; j < kOut; ++j)
                        a.y[(size_t)row * kOut + j] = (v[j] + __ldg(&a.b[3][j])) * __ldg(&a.out_scale[j]);
            }
        }
        if (s_fail[g]) break;
    }
    if (s_fail[g] && r == 0) atomicCAS(a.err, 0, a.err_code);
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_slot),
                     "r"(kTmemCols * kGroups)
                     : "memory");
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
    for (int l = 0; l < 4; ++l) {
        a.w[l] = d.wb[l];
        a.b[l] = d.b[l];
    }
    a.out_scale = d.out_scale;
    a.y = y;
    a.err = err;
    a.err_code = err_code;
    const int tiles = (n + kTileRows - 1) / kTileRows;
    const int per_cta = kGroups;
    const int want = (tiles + per_cta - 1) / per_cta;
    const int grid = want < n_sm ? want : n_sm;   // one CTA (4 warpgroups, 216 KB) per SM
    k_mlp_infer_tc<<<grid, 128 * kGroups, kSmemBytes, st>>>(a);
    count_launch();
    return cudaGetLastError();
}

}  // namespace sbs
