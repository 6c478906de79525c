// Host-side signed distance of a triangle mesh sampled on a grid, for
// environment bodies (what environment_body_t computes with Discregrid's
// MeshDistance, src/physics/environment_body.cpp:57-74).
//
// Distance: the closest point on each triangle by the Voronoi-region test of
// Ericson, "Real-Time Collision Detection" (2005), 5.1.5; the nearest
// triangle wins.  Sign: the angle-weighted pseudonormal of the closest
// feature (Baerentzen & Aanaes, "Signed distance computation using the angle
// weighted pseudonormal", IEEE TVCG 2005): the face normal inside a face, the
// sum of the adjacent faces' normals on an edge, the incidence-angle-weighted
// sum on a vertex; positive on the side the pseudonormal points to.  Faces are
// taken with their winding (b - a) x (c - a) pointing outside.  Brute force
// over triangles per node: O(nodes x triangles).
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <unordered_map>
#include <vector>

#include "../../include/sbs_gpu.h"

namespace {

struct V3 {
    double x, y, z;
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 unit(V3 a) {
    const double l = std::sqrt(dot(a, a));
    return l > 0 ? a * (1.0 / l) : a;
}

// feature: 0 face, 1 + k vertex k, 4 + k edge (k, k+1 mod 3)
struct Hit {
    double d2;
    V3 c;
    int feature;
};

Hit closest_on_triangle(V3 p, V3 a, V3 b, V3 c) {
    const V3 ab = b - a, ac = c - a, ap = p - a;
    const double d1 = dot(ab, ap), d2 = dot(ac, ap);
    auto done = [&](V3 q, int f) { const V3 d = p - q; return Hit{dot(d, d), q, f}; };
    if (d1 <= 0 && d2 <= 0) return done(a, 1);
    const V3 bp = p - b;
    const double d3 = dot(ab, bp), d4 = dot(ac, bp);
    if (d3 >= 0 && d4 <= d3) return done(b, 2);
    const double vc = d1 * d4 - d3 * d2;
    if (vc <= 0 && d1 >= 0 && d3 <= 0) return done(a + ab * (d1 / (d1 - d3)), 4);
    const V3 cp = p - c;
    const double d5 = dot(ab, cp), d6 = dot(ac, cp);
    if (d6 >= 0 && d5 <= d6) return done(c, 3);
    const double vb = d5 * d2 - d1 * d6;
    if (vb <= 0 && d2 >= 0 && d6 <= 0) return done(a + ac * (d2 / (d2 - d6)), 6);
    const double va = d3 * d6 - d5 * d4;
    if (va <= 0 && (d4 - d3) >= 0 && (d5 - d6) >= 0)
        return done(b + (c - b) * ((d4 - d3) / ((d4 - d3) + (d5 - d6))), 5);
    const double den = 1.0 / (va + vb + vc);
    return done(a + ab * (vb * den) + ac * (vc * den), 0);
}

inline uint64_t edge_key(uint32_t a, uint32_t b) {
    return a < b ? ((uint64_t)a << 32 | b) : ((uint64_t)b << 32 | a);
}

}  // namespace

namespace {

// Signed distance of a triangle mesh (pseudonormals precomputed), brute force
// over the triangles.
struct MeshSdf {
    std::vector<V3> x, fn, vn;
    std::unordered_map<uint64_t, V3> en;
    const uint32_t* tris;
    uint32_t n_tris;

    MeshSdf(const double* verts, uint32_t n_verts, const uint32_t* t, uint32_t nt) : tris(t), n_tris(nt) {
        x.resize(n_verts);
        for (uint32_t i = 0; i < n_verts; ++i) x[i] = {verts[3ull * i], verts[3ull * i + 1], verts[3ull * i + 2]};
        fn.resize(n_tris);
        vn.assign(n_verts, V3{0, 0, 0});
        for (uint32_t f = 0; f < n_tris; ++f) {
            const uint32_t* q = tris + 3ull * f;
            fn[f] = unit(cross(x[q[1]] - x[q[0]], x[q[2]] - x[q[0]]));
            for (int k = 0; k < 3; ++k) {
                const uint32_t v = q[k], v1 = q[(k + 1) % 3], v2 = q[(k + 2) % 3];
                const V3 e1 = unit(x[v1] - x[v]), e2 = unit(x[v2] - x[v]);
                const double ang = std::acos(std::max(-1.0, std::min(1.0, dot(e1, e2))));
                vn[v] = vn[v] + fn[f] * ang;
                auto it = en.find(edge_key(v, v1));
                if (it == en.end()) en.emplace(edge_key(v, v1), fn[f]);
                else it->second = it->second + fn[f];
            }
        }
    }

    double at(V3 p) {
        Hit best{1e300, {0, 0, 0}, 0};
        uint32_t bt = 0;
        for (uint32_t t = 0; t < n_tris; ++t) {
            const uint32_t* q = tris + 3ull * t;
            const Hit h = closest_on_triangle(p, x[q[0]], x[q[1]], x[q[2]]);
            if (h.d2 < best.d2) {
                best = h;
                bt = t;
            }
        }
        const uint32_t* q = tris + 3ull * bt;
        V3 n;
        if (best.feature == 0) n = fn[bt];
        else if (best.feature <= 3) n = vn[q[best.feature - 1]];
        else {
            const int e = best.feature - 4;
            n = en[edge_key(q[e], q[(e + 1) % 3])];
        }
        const double d = std::sqrt(best.d2);
        return dot(p - best.c, n) < 0 ? -d : d;
    }
};

sbs_status check_mesh(const double* verts, uint32_t n_verts, const uint32_t* tris, uint32_t n_tris, const double lo[3],
                      const double hi[3], const uint32_t cells[3], const float* values) {
    if (!verts || !tris || !lo || !hi || !cells || !values || n_verts == 0 || n_tris == 0) return SBS_EINVAL;
    for (int k = 0; k < 3; ++k)
        if (cells[k] == 0 || !(hi[k] > lo[k])) return SBS_EINVAL;
    for (uint64_t t = 0; t < 3ull * n_tris; ++t)
        if (tris[t] >= n_verts) return SBS_EINVAL;
    return SBS_OK;
}

}  // namespace

extern "C" sbs_status sbs_gpu_sdf_from_mesh(const double* verts, uint32_t n_verts, const uint32_t* tris,
                                            uint32_t n_tris, const double lo[3], const double hi[3],
                                            const uint32_t cells[3], float* values) {
    const sbs_status st = check_mesh(verts, n_verts, tris, n_tris, lo, hi, cells, values);
    if (st) return st;
    MeshSdf m(verts, n_verts, tris, n_tris);
    const uint32_t nx = cells[0] + 1, ny = cells[1] + 1, nz = cells[2] + 1;
    const double hx = (hi[0] - lo[0]) / cells[0], hy = (hi[1] - lo[1]) / cells[1], hz = (hi[2] - lo[2]) / cells[2];
    for (uint32_t k = 0; k < nz; ++k)
        for (uint32_t j = 0; j < ny; ++j)
            for (uint32_t i = 0; i < nx; ++i)
                values[((size_t)k * ny + j) * nx + i] = (float)m.at(V3{lo[0] + i * hx, lo[1] + j * hy, lo[2] + k * hz});
    return SBS_OK;
}

// The values of a cubic grid (layout of csrc/sdf_eval.cuh): the grid
// vertices, then the two nodes at 1/3 and 2/3 along every x-, y- and z-edge.
extern "C" sbs_status sbs_gpu_sdf_cubic_from_mesh(const double* verts, uint32_t n_verts, const uint32_t* tris,
                                                  uint32_t n_tris, const double lo[3], const double hi[3],
                                                  const uint32_t cells[3], float* values) {
    const sbs_status st = check_mesh(verts, n_verts, tris, n_tris, lo, hi, cells, values);
    if (st) return st;
    MeshSdf m(verts, n_verts, tris, n_tris);
    const uint64_t nx = cells[0] + 1, ny = cells[1] + 1, nz = cells[2] + 1;
    const double h[3] = {(hi[0] - lo[0]) / cells[0], (hi[1] - lo[1]) / cells[1], (hi[2] - lo[2]) / cells[2]};
    auto at = [&](double i, double j, double k) { return (float)m.at(V3{lo[0] + i * h[0], lo[1] + j * h[1], lo[2] + k * h[2]}); };
    size_t o = 0;
    for (uint64_t k = 0; k < nz; ++k)
        for (uint64_t j = 0; j < ny; ++j)
            for (uint64_t i = 0; i < nx; ++i) values[o++] = at(i, j, k);
    for (uint64_t k = 0; k < nz; ++k)
        for (uint64_t j = 0; j < ny; ++j)
            for (uint64_t i = 0; i + 1 < nx; ++i)
                for (int s = 0; s < 2; ++s) values[o++] = at(i + (s + 1) / 3.0, j, k);
    for (uint64_t k = 0; k < nz; ++k)
        for (uint64_t j = 0; j + 1 < ny; ++j)
            for (uint64_t i = 0; i < nx; ++i)
                for (int s = 0; s < 2; ++s) values[o++] = at(i, j + (s + 1) / 3.0, k);
    for (uint64_t k = 0; k + 1 < nz; ++k)
        for (uint64_t j = 0; j < ny; ++j)
            for (uint64_t i = 0; i < nx; ++i)
                for (int s = 0; s < 2; ++s) values[o++] = at(i, j, k + (s + 1) / 3.0);
    return SBS_OK;
}
