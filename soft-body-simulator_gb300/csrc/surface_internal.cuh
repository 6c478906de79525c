// Device copy of the bodies' visual models (surface_kernels.cu): the boundary
// triangle mesh that tetrahedral_mesh_boundary_t builds
// (src/physics/tetrahedral_mesh_boundary.cpp:76-120) and the per-vertex
// normals that compute_normals accumulates (:122-145).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sbs {

struct SurfaceDev {
    uint32_t* slot;       // [n_sv] device vertex slot of each surface vertex
    uint32_t* inc_start;  // [n_sv + 1] CSR of incident triangles
    uint32_t* inc;        // [3 n_tri] incident triangle ids, ascending per vertex
    uint4* tri;           // [n_tri] device vertex slots of the triangle's corners (w unused)
    float4* normal;       // [n_sv] normal state of the visual model (persists between updates)
    float* stage;         // [6 n_sv] position + normal records for copies to host memory
    uint32_t n_sv, n_tri;
};

// Updates surface vertices [sv0, sv0 + nsv): position = x of its vertex;
// normal = normalize((accumulate ? previous normal : 0) + sum over incident
// triangles, ascending, of (p2 - p1) x (p3 - p1)).  Writes position then
// normal into out[i * stride + 0..5] (i relative to sv0) when out != nullptr.
cudaError_t launch_surface_update(const SurfaceDev& sd, const float4* x, uint32_t sv0, uint32_t nsv, int accumulate,
                                  float* out, uint32_t stride, cudaStream_t st);

}  // namespace sbs
