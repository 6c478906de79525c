// State transfer between the caller's arrays (bodies in add order, vertices
// in input order, 3 floats each) and the library's layout (per-body Morton
// order, float4 with the inverse mass or the kinematic flag in .w): the
// permutation runs on the device, so a transfer is one copy each way.
#include <cuda_runtime.h>
#include <stdint.h>

#include "launch_count.cuh"
#include "xpbd_internal.cuh"

namespace sbs {

// out[3o..3o+2] = src[o2n[v0 + o]].xyz; *bad = 1 when check and a value is not finite
__global__ void k_gather_xyz(const float4* __restrict__ src, const uint32_t* __restrict__ o2n, uint32_t v0,
                             uint32_t nv, float* __restrict__ out, int check, int* bad) {
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < nv; o += gridDim.x * blockDim.x) {
        const float4 q = src[o2n[v0 + o]];
        out[3ull * o] = q.x;
        out[3ull * o + 1] = q.y;
        out[3ull * o + 2] = q.z;
        if (check && !(isfinite(q.x) && isfinite(q.y) && isfinite(q.z))) atomicExch(bad, 1);
    }
}

__global__ void k_check_finite(const float* __restrict__ in, uint64_t n, int* bad) {
    for (uint64_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        if (!isfinite(in[i])) atomicExch(bad, 1);
}

// dst[o2n[v0 + o]].xyz = in[3o..3o+2] (.w kept); also into dst2 when given.
// Nothing is written when skip is given and set (a failed input check ahead
// on the stream), so a rejected input leaves the state as it was.
__global__ void k_scatter_xyz(float4* __restrict__ dst, float4* __restrict__ dst2, const uint32_t* __restrict__ o2n,
                              uint32_t v0, uint32_t nv, const float* __restrict__ in, const int* skip) {
    if (skip && *skip) return;
    for (uint32_t o = blockIdx.x * blockDim.x + threadIdx.x; o < nv; o += gridDim.x * blockDim.x) {
        const uint32_t n = o2n[v0 + o];
        float4 q = dst[n];
        q.x = in[3ull * o];
        q.y = in[3ull * o + 1];
        q.z = in[3ull * o + 2];
        dst[n] = q;
        if (dst2) {
            float4 r = dst2[n];
            r.x = q.x; r.y = q.y; r.z = q.z;
            dst2[n] = r;
        }
    }
}

static int blocks(uint64_t n) {
    const uint64_t b = (n + 255) / 256;
    return (int)(b < 1 ? 1 : b > 4096 ? 4096 : b);
}

cudaError_t launch_gather_xyz(const float4* src, const uint32_t* o2n, uint32_t v0, uint32_t nv, float* out,
                              int check, int* bad, cudaStream_t st) {
    if (nv == 0) return cudaSuccess;
    k_gather_xyz<<<blocks(nv), 256, 0, st>>>(src, o2n, v0, nv, out, check, bad);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_check_finite(const float* in, uint64_t n, int* bad, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_check_finite<<<blocks(n), 256, 0, st>>>(in, n, bad);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_scatter_xyz(float4* dst, float4* dst2, const uint32_t* o2n, uint32_t v0, uint32_t nv,
                               const float* in, cudaStream_t st, const int* skip) {
    if (nv == 0) return cudaSuccess;
    k_scatter_xyz<<<blocks(nv), 256, 0, st>>>(dst, dst2, o2n, v0, nv, in, skip);
    count_launch();
    return cudaGetLastError();
}

}  // namespace sbs
