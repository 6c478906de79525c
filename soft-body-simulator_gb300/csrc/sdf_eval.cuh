// Signed-distance grids for environment bodies, evaluated with the
// interpolant's own gradient; a point outside the grid is outside the
// environment, as Discregrid reports the largest double there.
//  * cubic (the form environment_body_t builds with Discregrid's
//    CubicLagrangeDiscreteGrid, src/physics/environment_body.cpp:12-78, and
//    sdf_model_t::evaluate interpolates, src/physics/collision/sdf_model.cpp:66-75):
//    per cell the 32-node serendipity element of Koschier et al. 2017 ("An
//    hp-adaptive discretization algorithm for signed distance field
//    generation"): values at the 8 corners and at 2 points on each of the 12
//    edges (1/3 and 2/3 along it), shape functions on the reference cube
//    [-1, 1]^3
//      corner (sx, sy, sz) in {-1, 1}^3:
//        N = (1 + x sx)(1 + y sy)(1 + z sz)(9 (x^2 + y^2 + z^2) - 19) / 64
//      edge along x at x = t in {-1/3, 1/3}, (y, z) = (sy, sz):
//        N = 9/64 (1 - x^2)(1 + 9 x t)(1 + y sy)(1 + z sz)     (and cyclically),
//    which interpolate every cubic polynomial exactly.  Value layout: the
//    grid vertices (index (k * ny + j) * nx + i, nodes per axis n = cells + 1),
//    then two values per x-edge (index (k * ny + j) * (nx - 1) + i, the node
//    at 1/3 first), per y-edge ((k * (ny - 1) + j) * nx + i) and per z-edge
//    ((k * ny + j) * nx + i, k < nz - 1).
//  * trilinear: node values only (the grid vertices).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sbs {

constexpr int kMaxGrids = 2;

struct SdfGrid {
    const float* v;          // values (layout above)
    uint32_t nx, ny, nz;     // grid vertices per axis (>= 2)
    float ox, oy, oz;        // position of vertex (0, 0, 0)
    float hx, hy, hz;        // vertex spacing
    int cubic;               // 1: 32-node cubic cells, 0: trilinear
};

// Values a cubic grid with nx x ny x nz vertices holds.
__host__ __device__ __forceinline__ size_t sdf_cubic_count(uint32_t nx, uint32_t ny, uint32_t nz) {
    const size_t v = (size_t)nx * ny * nz;
    const size_t ex = (size_t)(nx - 1) * ny * nz, ey = (size_t)nx * (ny - 1) * nz, ez = (size_t)nx * ny * (nz - 1);
    return v + 2 * (ex + ey + ez);
}

// The 32-node cubic cell (i, j, k) at reference coordinates (x, y, z).
__host__ __device__ __forceinline__ void sdf_cubic_cell(const SdfGrid& g, uint32_t i, uint32_t j, uint32_t k, float x,
                                                        float y, float z, float& sd, float& dx, float& dy,
                                                        float& dz) {
    const size_t nx = g.nx, ny = g.ny, nz = g.nz;
    const size_t bx = nx * ny * nz, by = bx + 2 * (nx - 1) * ny * nz, bz = by + 2 * nx * (ny - 1) * nz;
    const float r2 = 9.0f * (x * x + y * y + z * z) - 19.0f;
    float f = 0.0f, fx = 0.0f, fy = 0.0f, fz = 0.0f;
    for (int c = 0; c < 8; ++c) {
        const int a = c & 1, b = (c >> 1) & 1, d = (c >> 2) & 1;
        const float sx = a ? 1.0f : -1.0f, sy = b ? 1.0f : -1.0f, sz = d ? 1.0f : -1.0f;
        const float v = g.v[((k + d) * ny + (j + b)) * nx + (i + a)];
        const float px = 1.0f + x * sx, py = 1.0f + y * sy, pz = 1.0f + z * sz;
        const float w = px * py * pz;
        f += v * w * r2;
        fx += v * (sx * py * pz * r2 + w * 18.0f * x);
        fy += v * (px * sy * pz * r2 + w * 18.0f * y);
        fz += v * (px * py * sz * r2 + w * 18.0f * z);
    }
    f *= 1.0f / 64.0f;
    fx *= 1.0f / 64.0f;
    fy *= 1.0f / 64.0f;
    fz *= 1.0f / 64.0f;
    // edge nodes: along axis `ax` at t = -1/3 (s = 0) or 1/3 (s = 1); the
    // other two coordinates at the cell's faces (e, h) in {-1, 1}
    const float q[3] = {x, y, z};
    for (int ax = 0; ax < 3; ++ax) {
        const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;
        const float u = q[ax], u1 = q[o1], u2 = q[o2];
        const float lu = 1.0f - u * u;
        for (int e = 0; e < 4; ++e) {
            const int b1 = e & 1, b2 = e >> 1;
            const float s1 = b1 ? 1.0f : -1.0f, s2 = b2 ? 1.0f : -1.0f;
            size_t base;
            if (ax == 0) base = bx + 2 * (((k + b2) * ny + (j + b1)) * (nx - 1) + i);
            else if (ax == 1) base = by + 2 * (((k + b2) * (ny - 1) + j) * nx + (i + b1));
            else base = bz + 2 * ((k * ny + (j + b2)) * nx + (i + b1));
            const float p1 = 1.0f + u1 * s1, p2 = 1.0f + u2 * s2;
            for (int sidx = 0; sidx < 2; ++sidx) {
                const float t = sidx ? (1.0f / 3.0f) : (-1.0f / 3.0f);
                const float v = g.v[base + sidx] * (9.0f / 64.0f);
                const float pt = 1.0f + 9.0f * u * t;
                const float w = lu * pt * p1 * p2;
                const float du = (-2.0f * u * pt + lu * 9.0f * t) * p1 * p2;
                const float d1 = lu * pt * s1 * p2, d2 = lu * pt * p1 * s2;
                f += v * w;
                const float dd[3] = {ax == 0 ? du : (o1 == 0 ? d1 : d2), ax == 1 ? du : (o1 == 1 ? d1 : d2),
                                     ax == 2 ? du : (o1 == 2 ? d1 : d2)};
                fx += v * dd[0];
                fy += v * dd[1];
                fz += v * dd[2];
            }
        }
    }
    sd = f;
    dx = fx;
    dy = fy;
    dz = fz;
}

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
    if (g.cubic) {
        float dx, dy, dz;
        sdf_cubic_cell(g, i, j, k, 2.0f * fx - 1.0f, 2.0f * fy - 1.0f, 2.0f * fz - 1.0f, sd, dx, dy, dz);
        gx = dx * 2.0f / g.hx;   // d/dp = d/dx * dx/dp, x = 2 (p - o) / h - 2 i - 1
        gy = dy * 2.0f / g.hy;
        gz = dz * 2.0f / g.hz;
        return true;
    }
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
