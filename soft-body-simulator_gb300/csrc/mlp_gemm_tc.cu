// The training GEMMs of the warm-start MLP on the 5th-generation tensor
// cores: forward products (rows x 128 x 16 or 128), input gradients
// (rows x 128 x 128 or 3) and split-K weight gradients (128 x 128 x batch).
//
// One CTA of 256 threads per 128 x 128 output tile (N padded to a multiple
// of 16 for the instruction's N), two CTAs per SM.  K advances in 64-column
// tiles through three shared-memory stages: all threads fill a stage (A and
// B rows; cp.async 16-byte copies, zero-filled past the matrix, where the
// operand is K-contiguous and aligned, element by element otherwise) in the
// canonical K-major layout of tc_common.cuh two tiles ahead of the tensor
// core; one thread issues up to four M = 128, K = 16 MMAs per stage into a
// TMEM accumulator of 128 FP32 columns and commits them to the stage's
// mbarrier, whose completion frees the stage for its next tile.  The
// epilogue reads the accumulator back with tcgen05.ld (warp w owns TMEM lanes
// 32 (w % 4).. and columns 64 (w / 4)..), applies bias / SiLU backward /
// SiLU, and writes the FP32 and BF16 outputs through a per-warp shared-memory
// transpose as 16-byte row segments; the transposed BF16 copy goes straight
// from the registers (a row of it is a column of the tile).
//
// Split-K slices write their partial products to a workspace that
// k_splitk_sum adds in slice order, so weight gradients are the same bit for
// bit on every run.  Every mbarrier wait is bounded in time; on expiry the
// kernel records an error code, frees its tensor memory and returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "launch_count.cuh"
#include "mlp_internal.cuh"
#include "tc_common.cuh"

namespace sbs {

namespace {

using namespace tc;

constexpr int kThreads = 256;                          // 8 warps: TMEM lane quarter x column half
constexpr int kTM = 128, kTN = 128, kTK = 64, kStages = 3;
constexpr uint32_t kTileA = kTM * kTK * 2;             // 16 KB
constexpr uint32_t kTileB = kTN * kTK * 2;             // 16 KB
constexpr uint32_t kStageBytes = kTileA + kTileB;
constexpr uint32_t kGemmSmem = kStages * kStageBytes;  // 96 KB: two CTAs per SM
constexpr uint32_t kTmemCols = 128;
constexpr unsigned long long kGemmWaitNs = 1000000000ull;  // 1 s
constexpr int kStageLd = 36;                           // epilogue transpose: 32 rows x 32 (+4) floats per warp
static_assert(8 * 32 * kStageLd * 4 <= (int)kGemmSmem, "epilogue staging fits in the operand stages");

// 16 bytes global -> shared, zero-filled beyond src_bytes (0 reads nothing)
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src), "r"(src_bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Rows [r0, r0 + nrows) x columns [k0, k0 + 8 kk8) of a 64-column canonical
// K-major tile at shared address dst (generic pointer dstp) from
// X(r, k) = X[r sr + k sk]; zero where r >= R or k >= kend.  Work items are
// (row, 8-column group) pairs ordered so that the eight lanes of a quarter
// warp fill the eight rows of one core matrix (128 contiguous bytes, no bank
// conflict) and four consecutive lanes read 64 contiguous bytes of one row.
// K-contiguous aligned operands (vec) go by cp.async, zero-filled past the
// matrix; others element by element.
__device__ __forceinline__ void fill_tile(uint32_t dst, uint8_t* dstp, const __nv_bfloat16* __restrict__ X,
                                          long long sr, long long sk, int r0, int R, int nrows, int k0, int kend,
                                          int kk8, bool vec) {
    const int items = nrows * 8;
    for (int it = (int)threadIdx.x; it < items; it += kThreads) {
        const int rr = (it >> 6) * 8 + (it & 7), k8 = (it >> 3) & 7;
        if (k8 >= kk8) continue;
        const int r = r0 + rr, k = k0 + k8 * 8;
        const uint32_t off = canon((uint32_t)rr, (uint32_t)(k8 * 8), kTK);
        if (vec) {
            const bool ok = r < R && k < kend;
            const uint32_t bytes = ok ? (uint32_t)min(8, kend - k) * 2u : 0u;
            cp_async16(dst + off, ok ? (const void*)(X + (long long)r * sr + k) : (const void*)X, bytes);
        } else {
            uint32_t w[4] = {0u, 0u, 0u, 0u};
            if (r < R) {
                const __nv_bfloat16* row = X + (long long)r * sr;
#pragma unroll
                for (int e = 0; e < 8; e += 2) {
                    const uint32_t lo = k + e < kend ? __bfloat16_as_ushort(row[(long long)(k + e) * sk]) : 0u;
                    const uint32_t hi = k + e + 1 < kend ? __bfloat16_as_ushort(row[(long long)(k + e + 1) * sk]) : 0u;
                    w[e / 2] = lo | (hi << 16);
                }
            }
            *reinterpret_cast<uint4*>(dstp + off) = make_uint4(w[0], w[1], w[2], w[3]);
        }
    }
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 p = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&p);
}

// The warp's 32 rows x 32 columns through its transpose buffer: lane = row
// writes its 32 values, then row segments go out whole.
__device__ __forceinline__ void stage_row(float* stage, const float (&v)[32]) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 8; ++q)
        *reinterpret_cast<float4*>(stage + lane * kStageLd + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
    __syncwarp();
}

// staged rows -> out[(row0 + r) * ld + col0 + c], c < ncols, row0 + r < M (FP32)
__device__ __forceinline__ void store_f32_rows(const float* stage, float* out, long long ld, int row0, int M,
                                               int col0, int ncols) {
    const int lane = threadIdx.x & 31;
    if (ncols == 32 && (ld & 3) == 0 && ((uintptr_t)out & 15) == 0 && (col0 & 3) == 0) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int r = i * 4 + (lane >> 3), c = 4 * (lane & 7);
            if (row0 + r < M)
                *reinterpret_cast<float4*>(out + (long long)(row0 + r) * ld + col0 + c) =
                    *reinterpret_cast<const float4*>(stage + r * kStageLd + c);
        }
    } else {
        for (int r = 0; r < 32; ++r)
            if (lane < ncols && row0 + r < M) out[(long long)(row0 + r) * ld + col0 + lane] = stage[r * kStageLd + lane];
    }
}

// the same as BF16
__device__ __forceinline__ void store_bf16_rows(const float* stage, __nv_bfloat16* out, long long ld, int row0,
                                                int M, int col0, int ncols) {
    const int lane = threadIdx.x & 31;
    if (ncols == 32 && (ld & 7) == 0 && ((uintptr_t)out & 15) == 0 && (col0 & 7) == 0) {
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int r = i * 8 + (lane >> 2), c = 8 * (lane & 3);
            const float4 a = *reinterpret_cast<const float4*>(stage + r * kStageLd + c);
            const float4 b = *reinterpret_cast<const float4*>(stage + r * kStageLd + c + 4);
            if (row0 + r < M)
                *reinterpret_cast<uint4*>(out + (long long)(row0 + r) * ld + col0 + c) =
                    make_uint4(pack_bf16(a.x, a.y), pack_bf16(a.z, a.w), pack_bf16(b.x, b.y), pack_bf16(b.z, b.w));
        }
    } else {
        for (int r = 0; r < 32; ++r)
            if (lane < ncols && row0 + r < M)
                out[(long long)(row0 + r) * ld + col0 + lane] = __float2bfloat16(stage[r * kStageLd + lane]);
    }
}

// in[(row0 + r) * ld + col0 + c] -> the transpose buffer (zero outside), then
// this lane's row into v
__device__ __forceinline__ void load_f32_rows(float* stage, const float* in, long long ld, int row0, int M, int col0,
                                              int ncols, float (&v)[32]) {
    const int lane = threadIdx.x & 31;
    __syncwarp();
    if (ncols == 32 && (ld & 3) == 0 && ((uintptr_t)in & 15) == 0 && (col0 & 3) == 0) {
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int r = i * 4 + (lane >> 3), c = 4 * (lane & 7);
            *reinterpret_cast<float4*>(stage + r * kStageLd + c) =
                row0 + r < M ? *reinterpret_cast<const float4*>(in + (long long)(row0 + r) * ld + col0 + c)
                             : make_float4(0.f, 0.f, 0.f, 0.f);
        }
    } else {
        for (int r = 0; r < 32; ++r)
            stage[r * kStageLd + lane] =
                (lane < ncols && row0 + r < M) ? in[(long long)(row0 + r) * ld + col0 + lane] : 0.0f;
    }
    __syncwarp();
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        const float4 f = *reinterpret_cast<const float4*>(stage + lane * kStageLd + 4 * q);
        v[4 * q] = f.x; v[4 * q + 1] = f.y; v[4 * q + 2] = f.z; v[4 * q + 3] = f.w;
    }
}

__global__ void __launch_bounds__(kThreads, 2) k_gemm_tc(GemmArgs g) {
    extern __shared__ __align__(1024) uint8_t sm[];
    __shared__ __align__(8) uint64_t mbar[kStages];
    __shared__ uint32_t tmem_slot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.x * kTM, n0 = blockIdx.y * kTN;
    const int bn = min(kTN, (g.N - n0 + 15) & ~15);   // instruction N: 16..128
    const int kper = g.splitk > 1 ? ((g.K + g.splitk * kTK - 1) / (g.splitk * kTK)) * kTK : g.K;
    const int kbeg = g.splitk > 1 ? (int)blockIdx.z * kper : 0;
    const int kend = g.splitk > 1 ? min(g.K, kbeg + kper) : g.K;
    const int nk = kend > kbeg ? (kend - kbeg + kTK - 1) / kTK : 0;
    const bool vec_a = g.sak == 1 && (g.sam & 7) == 0 && ((uintptr_t)g.A & 15) == 0;
    const bool vec_b = g.sbk == 1 && (g.sbn & 7) == 0 && ((uintptr_t)g.B & 15) == 0;

    if (warp == 0) tmem_alloc(smem_u32(&tmem_slot), kTmemCols);
    if (tid == 0) {
        for (int s = 0; s < kStages; ++s) mbar_init(smem_u32(&mbar[s]), 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = instr_desc(kTM, (uint32_t)bn);
    const uint32_t base = smem_u32(sm);
    auto issue = [&](int t) {
        const int s = t % kStages, k0 = kbeg + t * kTK;
        const int kk8 = 2 * min(kTK / 16, (kend - k0 + 15) / 16);
        fill_tile(base + s * kStageBytes, sm + s * kStageBytes, g.A, g.sam, g.sak, m0, g.M, kTM, k0, kend, kk8,
                  vec_a);
        fill_tile(base + s * kStageBytes + kTileA, sm + s * kStageBytes + kTileA, g.B, g.sbn, g.sbk, n0, g.N, bn, k0,
                  kend, kk8, vec_b);
    };
    // tiles 0 .. S-2 in flight before the first MMA; one cp.async group per tile
#pragma unroll
    for (int t = 0; t < kStages - 1; ++t) {
        if (t < nk) issue(t);
        cp_async_commit();
    }
    int fail = 0;
    for (int t = 0; t < nk; ++t) {
        const int s = t % kStages;
        cp_async_wait<kStages - 2>();   // this thread's copies of tile t have landed
        fence_async_smem();
        if (__syncthreads_or(fail)) {
            fail = 1;
            break;
        }
        if (tid == 0) {
            fence_after();
            const uint32_t a0 = base + s * kStageBytes, b0 = a0 + kTileA;
            const int nks = min(kTK / 16, (kend - (kbeg + t * kTK) + 15) / 16);
            for (int ks = 0; ks < nks; ++ks)
                mma(tmem, smem_desc(a0 + 256 * ks, kTK), smem_desc(b0 + 256 * ks, kTK), idesc,
                    (t > 0 || ks > 0) ? 1u : 0u);
            commit(smem_u32(&mbar[s]));
        }
        // refill the stage of tile t - 1 with tile t + S - 1 once tile t - 1's MMAs are done
        const int tn = t + kStages - 1;
        if (tn < nk) {
            if (t >= 1 &&
                !wait_phase(smem_u32(&mbar[(t - 1) % kStages]), (uint32_t)((t - 1) / kStages) & 1u, kGemmWaitNs))
                fail = 1;
            if (!fail) issue(tn);
        }
        cp_async_commit();
    }
    cp_async_wait<0>();
    // the tiles whose commits were not waited for above (MMAs complete in order)
    if (!fail)
        for (int t = max(0, nk - kStages); t < nk; ++t)
            if (!wait_phase(smem_u32(&mbar[t % kStages]), (uint32_t)(t / kStages) & 1u, kGemmWaitNs)) fail = 1;
    fail = __syncthreads_or(fail);
    fence_after();

    if (!fail) {
        // warp w: TMEM lanes (rows) 32 (w % 4).., columns 64 (w / 4)..
        const int q = warp & 3, hcol = (warp >> 2) * 64;
        float* stage = reinterpret_cast<float*>(sm) + warp * 32 * kStageLd;   // the operand stages are free now
        const int row0 = m0 + q * 32, m = row0 + lane;
        const uint32_t trow = tmem + (((uint32_t)q * 32u) << 16);
        for (int c0 = hcol; c0 < min(bn, hcol + 64); c0 += 32) {
            const int col0 = n0 + c0;
            const int ncols = min(32, g.N - col0);
            float v[32];
            if (nk > 0) {
                tmem_ld32(trow + (uint32_t)c0, v);
            } else {
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = 0.0f;
            }
            if (g.splitk > 1) {
                stage_row(stage, v);
                store_f32_rows(stage, g.ws + (long long)blockIdx.z * g.M * g.N, (long long)g.N, row0, g.M, col0, ncols);
                continue;
            }
            float z[32];
            if (g.dsilu) load_f32_rows(stage, g.dsilu, g.ldc, row0, g.M, col0, ncols, z);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int n = col0 + j;
                float x = v[j];
                if (g.beta != 0.0f && j < ncols && m < g.M) x += g.beta * g.C[(long long)m * g.ldc + n];
                if (g.bias && j < ncols) x += __ldg(&g.bias[n]);
                if (g.dsilu) x *= silu_grad(z[j]);
                v[j] = x;
            }
            if (g.C || g.Cb) {
                stage_row(stage, v);
                if (g.C) store_f32_rows(stage, g.C, g.ldc, row0, g.M, col0, ncols);
                if (g.Cb) store_bf16_rows(stage, g.Cb, g.ldc, row0, g.M, col0, ncols);
            }
            if (g.Act) {
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = silu(v[j]);
                stage_row(stage, v);
                store_bf16_rows(stage, g.Act, g.ldc, row0, g.M, col0, ncols);
            }
            if (g.T && m < g.M) {
                // a row of T is a column of the tile: lane = m writes 2 bytes, the warp 64 contiguous bytes
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (j < ncols) g.T[(long long)(col0 + j) * g.ldt + m] = __float2bfloat16(v[j]);
            }
        }
    } else if (tid == 0 && g.err) {
        atomicCAS(g.err, 0, g.err_code);
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        tmem_dealloc(tmem, kTmemCols);
    }
}

}  // namespace

cudaError_t gemm_tc(const GemmArgs& g, cudaStream_t st) {
    if (g.M <= 0 || g.N <= 0) return cudaSuccess;
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t e = cudaStreamIsCapturing(st, &cs);
    if (e != cudaSuccess) return e;
    if (cs == cudaStreamCaptureStatusNone &&
        (e = cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem)) !=
            cudaSuccess)
        return e;
    dim3 grid((g.M + kTM - 1) / kTM, (g.N + kTN - 1) / kTN, g.splitk > 1 ? g.splitk : 1);
    k_gemm_tc<<<grid, kThreads, kGemmSmem, st>>>(g);
    count_launch();
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (g.splitk > 1) return splitk_sum(g.ws, g.C, g.M * g.N, g.splitk, st);
    return cudaSuccess;
}

}  // namespace sbs
