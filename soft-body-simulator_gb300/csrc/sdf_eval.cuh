// Signed-distance grids for environment bodies: node samples of the signed
// distance on a regular grid, evaluated by trilinear interpolation with the
// interpolant's own gradient.  Stands in for the cubic Lagrange grid that
// environment_body_t builds with Discregrid (src/physics/environment_body.cpp:12-78,
// sdf_model_t::evaluate, src/physics/collision/sdf_model.cpp:66-75); a point
// outside the grid is outside the environment, as Discregrid reports the
// largest double there.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sbs {

constexpr int kMaxGrids = 2;

struct SdfGrid {
    const float* v;          // node values, index (k * ny + j) * nx + i
    uint32_t nx, ny, nz;     // nodes per axis (>= 2)
    float ox, oy, oz;        // position of node (0, 0, 0)
    float hx, hy, hz;        // node spacing
};

// Signed distance and gradient at p; false when p lies outside the grid.
__host__ __device__ __forceinline__ bool sdf_eval(const SdfGrid& g, float px, float py, float pz, float& sd,
                                                  float& gx, float& gy, float& gz) {
    const float u = (px - g.ox) / g.hx, w = (py - g.oy) / g.hy, t = (pz - g.oz) / g.hz;
    if (!(u >= 0.0f && w >= 0.0f && t >= 0.0f)) return false;
    if (!(u <= (float)(g.nx - 1) && w <= (float)(g.ny - 1) && t <= (float)(g.nz - 1))) return false;
    uint32_t i = (uint32_t)u, j = (uint32_t)w, k = (uint32_t)t;
    if (i > g.nx - 2) i = g.nx - 2;
    if (j > g.ny - 2) j = g.ny - 2;
    if (k > g.nz - 2) k = g.nz - 2;
    const float fx = u - (float)i, fy = w - (float)j, fz = t - (float)k;
    const size_t sx = 1, sy = g.nx, sz = (size_t)g.nx * g.ny;
    const size_t b = (size_t)k * sz + (size_t)j * sy + i;
    const float c000 = g.v[b], c100 = g.v[b + sx], c010 = g.v[b + sy], c110 = g.v[b + sx + sy];
    const float c001 = g.v[b + sz], c101 = g.v[b + sx + sz], c011 = g.v[b + sy + sz], c111 = g.v[b + sx + sy + sz];
    // along x, then y, then z
    const float c00 = c000 + fx * (c100 - c000), c10 = c010 + fx * (c110 - c010);
    const float c01 = c001 + fx * (c101 - c001), c11 = c011 + fx * (c111 - c011);
    const float c0 = c00 + fy * (c10 - c00), c1 = c01 + fy * (c11 - c01);
    sd = c0 + fz * (c1 - c0);
    // derivatives of the interpolant, in world units
    const float dx00 = c100 - c000, dx10 = c110 - c010, dx01 = c101 - c001, dx11 = c111 - c011;
    const float dx0 = dx00 + fy * (dx10 - dx00), dx1 = dx01 + fy * (dx11 - dx01);
    gx = (dx0 + fz * (dx1 - dx0)) / g.hx;
    const float dy0 = c10 - c00, dy1 = c11 - c01;
    gy = (dy0 + fz * (dy1 - dy0)) / g.hy;
    gz = (c1 - c0) / g.hz;
    return true;
}

}  // namespace sbs
