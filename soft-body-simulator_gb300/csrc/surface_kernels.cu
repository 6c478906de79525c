// Visual-model update on the device: tetrahedral_body_t::update_visual_model
// (src/physics/tetrahedral_body.cpp:157-165) copies each surface vertex's
// position from its particle and calls compute_normals
// (src/physics/tetrahedral_mesh_boundary.cpp:122-145), which adds every
// boundary triangle's unnormalised normal (p2 - p1) x (p3 - p1) to its three
// vertices in triangle order and then normalises each vertex normal.  The
// vertex normals are never cleared there, so each update adds to the previous
// (normalised) normal; `accumulate` keeps that behaviour, 0 starts from zero.
//
// One thread per surface vertex gathers its incident triangles in ascending
// order, so every vertex sums the same terms in the same order as the
// sequential scatter loop, with no atomics.
#include <cuda_runtime.h>
#include <stdint.h>

#include "surface_internal.cuh"
#include "launch_count.cuh"

namespace sbs {

__global__ void k_surface_update(SurfaceDev sd, const float4* __restrict__ x, uint32_t sv0, uint32_t nsv,
                                 int accumulate, float* __restrict__ out, uint32_t stride) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nsv; i += gridDim.x * blockDim.x) {
        const uint32_t sv = sv0 + i;
        float nx = 0.f, ny = 0.f, nz = 0.f;
        if (accumulate) {
            const float4 n0 = sd.normal[sv];
            nx = n0.x; ny = n0.y; nz = n0.z;
        }
        const uint32_t b = sd.inc_start[sv], e = sd.inc_start[sv + 1];
        for (uint32_t k = b; k < e; ++k) {
            const uint4 t = sd.tri[sd.inc[k]];
            const float4 p1 = x[t.x], p2 = x[t.y], p3 = x[t.z];
            const float ax = p2.x - p1.x, ay = p2.y - p1.y, az = p2.z - p1.z;
            const float bx = p3.x - p1.x, by = p3.y - p1.y, bz = p3.z - p1.z;
            nx += ay * bz - az * by;
            ny += az * bx - ax * bz;
            nz += ax * by - ay * bx;
        }
        // normalise when the squared norm is positive, else leave unchanged
        const float z = nx * nx + ny * ny + nz * nz;
        if (z > 0.0f) {
            const float r = __fsqrt_rn(z);
            nx = __fdiv_rn(nx, r);
            ny = __fdiv_rn(ny, r);
            nz = __fdiv_rn(nz, r);
        }
        sd.normal[sv] = make_float4(nx, ny, nz, 0.0f);
        if (out) {
            const float4 p = x[sd.slot[sv]];
            float* o = out + (size_t)i * stride;
            o[0] = p.x; o[1] = p.y; o[2] = p.z;
            o[3] = nx; o[4] = ny; o[5] = nz;
        }
    }
}

cudaError_t launch_surface_update(const SurfaceDev& sd, const float4* x, uint32_t sv0, uint32_t nsv, int accumulate,
                                  float* out, uint32_t stride, cudaStream_t st) {
    if (nsv == 0) return cudaSuccess;
    const uint32_t grid = (nsv + 255) / 256 < 4096u ? (nsv + 255) / 256 : 4096u;
    k_surface_update<<<grid, 256, 0, st>>>(sd, x, sv0, nsv, accumulate, out, stride);
    count_launch();
    return cudaGetLastError();
}

}  // namespace sbs
