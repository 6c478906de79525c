// FP64 CPU oracle for the XPBD substep loop.
//
// TEST INFRASTRUCTURE ONLY.  The CUDA library's results are checked against
// it: it is loaded by tests/, by __graft_entry__.smoke() and by bench.py's CPU
// baseline arm, never by the product path.
//
// It restates, in plain C++17 with no dependencies, the reference's
// sequential XPBD loop (Q-Minh/soft-body-simulator):
//   * timestep_t::step                 src/physics/timestep.cpp:20-70
//   * gauss_seidel_solver_t::solve     src/physics/gauss_seidel_solver.cpp:8-37
//   * constraint_t::prepare_for_projection  src/physics/constraint.cpp:12-16
//   * green_constraint_t (ctor + project_positions + signed_volume)
//                                      src/physics/xpbd/green_constraint.cpp:11-173
//   * collision_constraint_t           src/physics/xpbd/collision_constraint.cpp:21-48
//   * plane contacts on surface vertices  src/physics/collision/bvh_model.cpp:72-94,
//                                      sdf_model.cpp:52-64, contact_handler.cpp:14-54
//   * particle_t::invmass / a()        src/physics/particle.cpp:39-53
//   * distance_constraint_t            src/physics/xpbd/distance_constraint.cpp:8-53
//   * the visual model's boundary mesh and normals
//                                      src/physics/tetrahedral_mesh_boundary.cpp:76-145,
//                                      src/physics/tetrahedral_body.cpp:157-165
// with the same data structure the reference uses: an array of particle
// records (x0, xi, xn, x, v, f, m) and a list of constraint objects projected
// through a virtual call, one at a time, in list order.
//
// Additions the reference does not have (each marked where it is written):
// stable Neo-Hookean constraints (Macklin & Mueller 2021), lumped masses,
// gravity as an acceleration, kinematic (prescribed) vertices, an external
// acceleration field, body-body vertex-in-tet contacts from a CPU spatial
// hash, the XPBD residual and energy, and a hook that permutes the elastic
// constraint list into the GPU's colour order so both run the same sweep.
// An optional thread count runs each colour's (vertex-disjoint) constraints
// in parallel; the arithmetic per constraint is unchanged, so the result is
// bit-identical to the sequential sweep.
//
// Parity status: the reference cannot be compiled here (Eigen, Discregrid and
// the GL stack are absent) and ships no tests or golden vectors, so this
// oracle is "parity unpinned" against reference outputs.  It is cross-checked
// against an independent numpy restatement (oracle/numpy_oracle.py, which
// uses LAPACK's SVD in place of the Jacobi SVD below) and against analytic
// known answers of the reference's formulas.
//
// The 3x3 SVD: Eigen's JacobiSVD is third-party and not in the reference
// tree; here it is a one-sided (Hestenes) Jacobi SVD written from the textbook
// method (Golub & Van Loan, "Matrix Computations", 8.6.3), returning Eigen's
// documented convention: singular values >= 0, sorted in decreasing order.

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace orc {

struct vec3 {
    double x = 0, y = 0, z = 0;
    vec3() = default;
    vec3(double a, double b, double c) : x(a), y(b), z(c) {}
    double& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    double operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
static inline vec3 operator+(vec3 a, vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline vec3 operator-(vec3 a, vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline vec3 operator-(vec3 a) { return {-a.x, -a.y, -a.z}; }
static inline vec3 operator*(vec3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
static inline vec3 operator*(double s, vec3 a) { return {a.x * s, a.y * s, a.z * s}; }
static inline vec3 operator/(vec3 a, double s) { return {a.x / s, a.y / s, a.z / s}; }
static inline vec3& operator+=(vec3& a, vec3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
static inline double dot(vec3 a, vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline vec3 cross(vec3 a, vec3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline double norm(vec3 a) { return std::sqrt(dot(a, a)); }

// 3x3 matrix, row-major m[r][c].
struct mat3 {
    double m[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    static mat3 identity() { mat3 r; r.m[0][0] = r.m[1][1] = r.m[2][2] = 1; return r; }
    static mat3 from_cols(vec3 a, vec3 b, vec3 c) {
        mat3 r;
        for (int i = 0; i < 3; ++i) { r.m[i][0] = a[i]; r.m[i][1] = b[i]; r.m[i][2] = c[i]; }
        return r;
    }
    vec3 col(int c) const { return {m[0][c], m[1][c], m[2][c]}; }
    void set_col(int c, vec3 v) { m[0][c] = v.x; m[1][c] = v.y; m[2][c] = v.z; }
    mat3 T() const { mat3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = m[j][i]; return r; }
    double det() const {
        return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
               m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
               m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    }
    double trace() const { return m[0][0] + m[1][1] + m[2][2]; }
};
static inline mat3 operator*(const mat3& a, const mat3& b) {
    mat3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            r.m[i][j] = a.m[i][0] * b.m[0][j] + a.m[i][1] * b.m[1][j] + a.m[i][2] * b.m[2][j];
    return r;
}
static inline mat3 operator*(const mat3& a, double s) {
    mat3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] * s; return r;
}
static inline mat3 operator+(const mat3& a, const mat3& b) {
    mat3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] + b.m[i][j]; return r;
}
static inline mat3 operator-(const mat3& a, const mat3& b) {
    mat3 r; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) r.m[i][j] = a.m[i][j] - b.m[i][j]; return r;
}
static inline mat3 inverse(const mat3& a) {
    double d = a.det();
    mat3 r;
    r.m[0][0] = (a.m[1][1] * a.m[2][2] - a.m[1][2] * a.m[2][1]) / d;
    r.m[0][1] = (a.m[0][2] * a.m[2][1] - a.m[0][1] * a.m[2][2]) / d;
    r.m[0][2] = (a.m[0][1] * a.m[1][2] - a.m[0][2] * a.m[1][1]) / d;
    r.m[1][0] = (a.m[1][2] * a.m[2][0] - a.m[1][0] * a.m[2][2]) / d;
    r.m[1][1] = (a.m[0][0] * a.m[2][2] - a.m[0][2] * a.m[2][0]) / d;
    r.m[1][2] = (a.m[0][2] * a.m[1][0] - a.m[0][0] * a.m[1][2]) / d;
    r.m[2][0] = (a.m[1][0] * a.m[2][1] - a.m[1][1] * a.m[2][0]) / d;
    r.m[2][1] = (a.m[0][1] * a.m[2][0] - a.m[0][0] * a.m[2][1]) / d;
    r.m[2][2] = (a.m[0][0] * a.m[1][1] - a.m[0][1] * a.m[1][0]) / d;
    return r;
}
static inline double frob2(const mat3& a) {
    double s = 0; for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) s += a.m[i][j] * a.m[i][j]; return s;
}

// One-sided Jacobi SVD: F = U diag(s) V^T, s >= 0 descending.
void svd3(const mat3& F, mat3& U, vec3& s, mat3& V) {
    vec3 a[3] = {F.col(0), F.col(1), F.col(2)};
    vec3 v[3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
    for (int sweep = 0; sweep < 60; ++sweep) {
        bool rotated = false;
        for (auto& pq : pairs) {
            int p = pq[0], q = pq[1];
            double alpha = dot(a[p], a[p]), beta = dot(a[q], a[q]), gamma = dot(a[p], a[q]);
            if (std::fabs(gamma) <= 1e-15 * std::sqrt(alpha * beta) || gamma == 0.0) continue;
            rotated = true;
            double zeta = (beta - alpha) / (2.0 * gamma);
            double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
            double c = 1.0 / std::sqrt(1.0 + t * t), sn = c * t;
            vec3 ap = a[p], aq = a[q];
            a[p] = c * ap - sn * aq;
            a[q] = sn * ap + c * aq;
            vec3 vp = v[p], vq = v[q];
            v[p] = c * vp - sn * vq;
            v[q] = sn * vp + c * vq;
        }
        if (!rotated) break;
    }
    double sig[3] = {norm(a[0]), norm(a[1]), norm(a[2])};
    int idx[3] = {0, 1, 2};
    std::sort(idx, idx + 3, [&](int i, int j) { return sig[i] > sig[j]; });
    vec3 u[3];
    double maxs = std::max(sig[idx[0]], 1e-300);
    bool ok[3];
    for (int k = 0; k < 3; ++k) {
        int i = idx[k];
        s[k] = sig[i];
        V.set_col(k, v[i]);
        ok[k] = sig[i] > 1e-13 * maxs && sig[i] > 1e-300;
        u[k] = ok[k] ? a[i] / sig[i] : vec3{};
    }
    // Complete U for (numerically) zero singular values.
    if (!ok[0]) { u[0] = {1, 0, 0}; }
    if (!ok[1]) {
        vec3 e = std::fabs(u[0].x) < 0.9 ? vec3{1, 0, 0} : vec3{0, 1, 0};
        vec3 w = e - u[0] * dot(e, u[0]);
        u[1] = w / norm(w);
    }
    if (!ok[2]) u[2] = cross(u[0], u[1]);
    for (int k = 0; k < 3; ++k) U.set_col(k, u[k]);
}

// ---------------------------------------------------------------------------
// State: particle_t restated from include/sbs/physics/particle.h:45-52.
struct particle_t {
    vec3 x0, xi, xn, x, v, f;
    double m = 1.0;
    // additions: prescribed motion and a body acceleration field
    int kin = -1;        // index into sim.kinematics, -1 if free
    vec3 ext_acc;
    double invmass() const { return m > 0.0 ? 1.0 / m : 0.0; }   // particle.cpp:39-44
    vec3 a() const { return f * invmass(); }                       // particle.cpp:50-53
};

struct sim_t;

// constraint_t restated from include/sbs/physics/constraint.h:12-35.
struct constraint_t {
    double alpha, beta, lagrange = 0.0;
    constraint_t(double a, double b) : alpha(a), beta(b) {}
    virtual ~constraint_t() = default;
    virtual void prepare_for_projection() { lagrange = 0.0; }
    virtual void project_positions(sim_t& sim, double dt) = 0;
    // sum of (C + alpha~ lambda)^2 and the elastic energy at the current xi
    virtual void residual(const sim_t& sim, double dt, double& r2, double& energy) const = 0;
};

struct kinematic_t {
    vec3 center, axis;
    double omega;
};

struct plane_t { vec3 n; double d; };

// Signed-distance grid of an environment body.  cubic: the reference's
// Discregrid cubic Lagrange grid (sdf_model.cpp:66-75, environment_body.cpp:
// 72-73), per cell the 32-node serendipity element (Koschier et al. 2017):
// corner values and values at 1/3 and 2/3 of every edge (value layout: the
// (cells+1)^3 vertices, then two per x-, y- and z-edge); otherwise node values
// with trilinear interpolation.  The gradient is the interpolant's.
struct grid_t {
    std::vector<double> v;
    uint32_t n[3];
    double o[3], h[3];
    bool cubic = false;

    // the 32-node cell (c0, c1, c2) at reference coordinates r in [-1, 1]^3:
    // value and derivatives w.r.t. r
    void cubic_cell(const uint32_t c[3], const double r[3], double& f, double d[3]) const {
        const size_t nx = n[0], ny = n[1], nz = n[2];
        const size_t base[3] = {nx * ny * nz, nx * ny * nz + 2 * (nx - 1) * ny * nz,
                                nx * ny * nz + 2 * (nx - 1) * ny * nz + 2 * nx * (ny - 1) * nz};
        f = 0.0;
        d[0] = d[1] = d[2] = 0.0;
        const double q = 9.0 * (r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) - 19.0;
        for (int a = 0; a < 2; ++a)
            for (int b = 0; b < 2; ++b)
                for (int e = 0; e < 2; ++e) {
                    const double s[3] = {a ? 1.0 : -1.0, b ? 1.0 : -1.0, e ? 1.0 : -1.0};
                    const double val = v[((c[2] + e) * ny + (c[1] + b)) * nx + (c[0] + a)] / 64.0;
                    const double l[3] = {1 + r[0] * s[0], 1 + r[1] * s[1], 1 + r[2] * s[2]};
                    f += val * l[0] * l[1] * l[2] * q;
                    for (int k = 0; k < 3; ++k) {
                        const double lk = l[(k + 1) % 3] * l[(k + 2) % 3];
                        d[k] += val * (s[k] * lk * q + l[0] * l[1] * l[2] * 18.0 * r[k]);
                    }
                }
        for (int ax = 0; ax < 3; ++ax) {
            const int o1 = (ax + 1) % 3, o2 = (ax + 2) % 3;
            for (int b1 = 0; b1 < 2; ++b1)
                for (int b2 = 0; b2 < 2; ++b2) {
                    uint32_t g[3] = {c[0], c[1], c[2]};
                    g[o1] += b1;
                    g[o2] += b2;
                    size_t idx;
                    if (ax == 0) idx = base[0] + 2 * ((g[2] * ny + g[1]) * (nx - 1) + g[0]);
                    else if (ax == 1) idx = base[1] + 2 * ((g[2] * (ny - 1) + g[1]) * nx + g[0]);
                    else idx = base[2] + 2 * ((g[2] * ny + g[1]) * nx + g[0]);
                    const double s1 = b1 ? 1.0 : -1.0, s2 = b2 ? 1.0 : -1.0;
                    const double p1 = 1 + r[o1] * s1, p2 = 1 + r[o2] * s2, u = r[ax];
                    for (int t = 0; t < 2; ++t) {
                        const double tt = t ? 1.0 / 3.0 : -1.0 / 3.0;
                        const double val = v[idx + t] * 9.0 / 64.0;
                        const double pu = (1 - u * u) * (1 + 9 * u * tt);
                        f += val * pu * p1 * p2;
                        d[ax] += val * (-2 * u * (1 + 9 * u * tt) + (1 - u * u) * 9 * tt) * p1 * p2;
                        d[o1] += val * pu * s1 * p2;
                        d[o2] += val * pu * p1 * s2;
                    }
                }
        }
    }

    // false outside the grid (no contact there)
    bool eval(vec3 p, double& sd, vec3& g) const {
        const double u[3] = {(p.x - o[0]) / h[0], (p.y - o[1]) / h[1], (p.z - o[2]) / h[2]};
        uint32_t c[3];
        double f[3];
        for (int k = 0; k < 3; ++k) {
            if (!(u[k] >= 0.0 && u[k] <= (double)(n[k] - 1))) return false;
            c[k] = std::min((uint32_t)u[k], n[k] - 2);
            f[k] = u[k] - c[k];
        }
        if (cubic) {
            const double r[3] = {2 * f[0] - 1, 2 * f[1] - 1, 2 * f[2] - 1};
            double d[3];
            cubic_cell(c, r, sd, d);
            g = {d[0] * 2 / h[0], d[1] * 2 / h[1], d[2] * 2 / h[2]};
            return true;
        }
        auto at = [&](uint32_t i, uint32_t j, uint32_t k) {
            return v[((size_t)(c[2] + k) * n[1] + (c[1] + j)) * n[0] + (c[0] + i)];
        };
        double w[2][2][2];
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) w[i][j][k] = at(i, j, k);
        const double fx = f[0], fy = f[1], fz = f[2];
        sd = 0.0;
        g = {0.0, 0.0, 0.0};
        for (int i = 0; i < 2; ++i)
            for (int j = 0; j < 2; ++j)
                for (int k = 0; k < 2; ++k) {
                    const double bx = i ? fx : 1 - fx, by = j ? fy : 1 - fy, bz = k ? fz : 1 - fz;
                    sd += w[i][j][k] * bx * by * bz;
                    g.x += w[i][j][k] * (i ? 1.0 : -1.0) * by * bz / h[0];
                    g.y += w[i][j][k] * bx * (j ? 1.0 : -1.0) * bz / h[1];
                    g.z += w[i][j][k] * bx * by * (k ? 1.0 : -1.0) / h[2];
                }
        return true;
    }
};

struct body_t {
    uint32_t v0, nv, t0, nt;
    std::vector<uint32_t> surface;   // global vertex ids, ascending
    std::vector<std::array<uint32_t, 3>> surface_tris;  // global ids, outward
    int model;
    // visual model (tetrahedral_mesh_boundary_t): triangles in surface-local
    // ids, surface vertex -> global particle, accumulated vertex normals
    std::vector<std::array<uint32_t, 3>> vis_tris;
    std::vector<uint32_t> vis_map;
    std::vector<vec3> vis_normal;
};

// tetrahedral_body_t::update_visual_model (src/physics/tetrahedral_body.cpp:157-165)
// followed by compute_normals (src/physics/tetrahedral_mesh_boundary.cpp:122-145):
// positions from the particles' x; every boundary triangle adds
// (p2 - p1) x (p3 - p1) to its three vertex normals, in triangle order; then
// each normal is normalised (left unchanged when its squared norm is 0, as
// Eigen's normalize() does).  The normals are not cleared first.
static void update_visual_model(const std::vector<particle_t>& particles, body_t& b, std::vector<vec3>* pos) {
    if (pos) {
        pos->resize(b.vis_map.size());
        for (size_t i = 0; i < b.vis_map.size(); ++i) (*pos)[i] = particles[b.vis_map[i]].x;
    }
    for (const auto& t : b.vis_tris) {
        const vec3 p1 = particles[b.vis_map[t[0]]].x, p2 = particles[b.vis_map[t[1]]].x,
                   p3 = particles[b.vis_map[t[2]]].x;
        const vec3 n = cross(p2 - p1, p3 - p1);
        b.vis_normal[t[0]] += n;
        b.vis_normal[t[1]] += n;
        b.vis_normal[t[2]] += n;
    }
    for (auto& n : b.vis_normal) {
        const double z = dot(n, n);
        if (z > 0.0) n = n / std::sqrt(z);
    }
}

struct params_t {
    double alpha = 1e-4, beta = 0.0, collision_alpha = 1e-8;
    vec3 gravity{0.0, -9.81, 0.0};
    int gravity_mode = 0;   // 0 acceleration (m g as force), 1 force as in timestep.cpp:39
    double hash_cell = 0.0;
    int body_contacts = 0;  // 1: vertex-in-tet contacts between bodies, 2: also within a body
};

// Per-tet topology for the spatial hash (global vertex ids, add order).
struct tet_topo_t {
    uint32_t v[4];
    uint32_t body;
    uint8_t bmask;   // bit f: face f of faces_copy (topology.cpp:335-342) is on the boundary
};

struct stats_t {
    double residual = 0, energy = 0, r2_elastic = 0, r2_contact = 0;
    uint64_t projections = 0;
    uint32_t n_contacts = 0, n_body_contacts = 0;
};

struct sim_t {
    params_t prm;
    std::vector<particle_t> particles;
    std::vector<body_t> bodies;
    std::vector<std::unique_ptr<constraint_t>> constraints;            // elastic, global tet order
    std::vector<constraint_t*> sweep;                                  // permuted projection order
    std::vector<uint32_t> colour_offsets;                              // optional, into sweep
    std::vector<std::unique_ptr<constraint_t>> collision_constraints;  // rebuilt every frame
    std::vector<uint32_t> ground_end;                                  // ground contacts per plane
    std::vector<kinematic_t> kinematics;
    std::vector<plane_t> planes;
    std::vector<grid_t> grids;              // environment slots after the planes
    std::vector<tet_topo_t> topo;          // global tet order
    std::vector<uint32_t> vbody;           // per particle
    std::vector<uint8_t> vsurf;            // per particle: surface vertex
    std::vector<uint32_t> slot_of_tet;     // sweep slot of each tet (tie-breaks)
    // distance constraints, input order; projected after the tets in
    // edge_order (colour-major), with their colour boundaries in edge_offsets
    std::vector<std::unique_ptr<constraint_t>> edges;
    std::vector<uint32_t> edge_order, edge_offsets;
    double time = 0.0;
    int threads = 1;
    stats_t st;
    std::vector<double> residual_history;   // per iteration, when enabled
    int record_history = 0;
};

// ---------------------------------------------------------------------------
// green_constraint_t: src/physics/xpbd/green_constraint.cpp:11-173
struct green_constraint_t final : constraint_t {
    uint32_t v[4];
    mat3 DmInv;
    double V0, mu, lambda;

    green_constraint_t(double a, double b, const sim_t& sim, const uint32_t* vi, double E, double nu)
        : constraint_t(a, b) {
        for (int i = 0; i < 4; ++i) v[i] = vi[i];
        const auto& p = sim.particles;
        mat3 Dm = mat3::from_cols(p[v[0]].x0 - p[v[3]].x0, p[v[1]].x0 - p[v[3]].x0,
                                  p[v[2]].x0 - p[v[3]].x0);
        DmInv = inverse(Dm);
        V0 = (1.0 / 6.0) * Dm.det();
        mu = E / (2.0 * (1.0 + nu));
        lambda = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu));
    }

    static double signed_volume(vec3 p1, vec3 p2, vec3 p3, vec3 p4) {
        return (1.0 / 6.0) * mat3::from_cols(p1 - p4, p2 - p4, p3 - p4).det();
    }

    // Steps 2-8 of project_positions: psi and the four gradients f_i
    // (f = -grad C), evaluated at xi.
    void evaluate(const sim_t& sim, double& psi, vec3 f[4]) const {
        const auto& P = sim.particles;
        vec3 x1 = P[v[0]].xi, x2 = P[v[1]].xi, x3 = P[v[2]].xi, x4 = P[v[3]].xi;
        double Vs = signed_volume(x1, x2, x3, x4);
        bool Vpos = Vs >= 0.0, V0pos = V0 >= 0.0;
        bool inverted = (Vpos && !V0pos) || (!Vpos && V0pos);
        mat3 Ds = mat3::from_cols(x1 - x4, x2 - x4, x3 - x4);
        mat3 F = Ds * DmInv;
        mat3 U, Vm; vec3 sg;
        svd3(F, U, sg, Vm);
        mat3 Fhat;
        Fhat.m[0][0] = sg[0]; Fhat.m[1][1] = sg[1]; Fhat.m[2][2] = sg[2];
        if (inverted) {
            Fhat.m[2][2] = -Fhat.m[2][2];
            U.set_col(2, -U.col(2));
        }
        const double min_sv = 0.577;
        for (int i = 0; i < 3; ++i) Fhat.m[i][i] = std::max(Fhat.m[i][i], min_sv);
        mat3 I = mat3::identity();
        mat3 Ehat = (Fhat.T() * Fhat - I) * 0.5;
        double EhatTrace = Ehat.trace();
        mat3 Phat = Fhat * (Ehat * (2.0 * mu) + I * (lambda * EhatTrace));
        mat3 E = U * Ehat * Vm.T();     // as written in the reference (U, not V)
        double Etr = E.trace();
        psi = mu * frob2(E) + 0.5 * lambda * Etr * Etr;
        mat3 Piola = U * Phat * Vm.T();
        double aV0 = std::fabs(V0);
        mat3 H = Piola * DmInv.T() * (-aV0);
        f[0] = H.col(0); f[1] = H.col(1); f[2] = H.col(2);
        f[3] = -(f[0] + f[1] + f[2]);
    }

    void project_positions(sim_t& sim, double dt) override {
        auto& P = sim.particles;
        double w[4];
        for (int i = 0; i < 4; ++i) w[i] = P[v[i]].invmass();
        double psi; vec3 f[4];
        evaluate(sim, psi, f);
        double S = 0;
        for (int i = 0; i < 4; ++i) S += w[i] * dot(f[i], f[i]);
        const double epsilon = 1e-20;
        if (S < epsilon) return;
        double C = std::fabs(V0) * psi;
        double dt2 = dt * dt;
        double at = alpha / dt2, bt = beta * dt2, gamma = at * bt / dt;
        double gd = 0;
        for (int i = 0; i < 4; ++i) gd += dot(f[i], P[v[i]].xi - P[v[i]].xn);
        double num = -(C + at * lagrange) + gamma * gd;
        double den = (1.0 + gamma) * S + at;
        double dl = num / den;
        lagrange += dl;
        for (int i = 0; i < 4; ++i) P[v[i]].xi += (w[i] * -f[i]) * dl;
    }

    void residual(const sim_t& sim, double dt, double& r2, double& energy) const override {
        double psi; vec3 f[4];
        evaluate(sim, psi, f);
        double C = std::fabs(V0) * psi;
        double h = C + alpha / (dt * dt) * lagrange;
        r2 += h * h;
        energy += C;
    }
};

// ---------------------------------------------------------------------------
// Stable Neo-Hookean tet (Macklin & Mueller 2021, "A Constraint-based
// Formulation of Stable Neo-Hookean Materials"): deviatoric C_D = ||F||_F with
// compliance 1/(mu |V0|) and hydrostatic C_H = det F - (1 + mu/lambda) with
// compliance 1/(lambda |V0|), each with its own multiplier, solved together
// as the paper's coupled 2x2 system.  (Solving them one after the other with
// multipliers reset every substep drifts away from the rest state, because
// C_D is not zero at rest.)  Not in the reference.
struct snh_constraint_t final : constraint_t {
    uint32_t v[4];
    mat3 DmInv;
    double V0, mu, lambda, lagrange_h = 0.0;

    snh_constraint_t(const sim_t& sim, const uint32_t* vi, double E, double nu) : constraint_t(0, 0) {
        for (int i = 0; i < 4; ++i) v[i] = vi[i];
        const auto& p = sim.particles;
        mat3 Dm = mat3::from_cols(p[v[0]].x0 - p[v[3]].x0, p[v[1]].x0 - p[v[3]].x0,
                                  p[v[2]].x0 - p[v[3]].x0);
        DmInv = inverse(Dm);
        V0 = (1.0 / 6.0) * Dm.det();
        mu = E / (2.0 * (1.0 + nu));
        lambda = (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu));
    }
    void prepare_for_projection() override { lagrange = 0.0; lagrange_h = 0.0; }

    mat3 deformation(const sim_t& sim) const {
        const auto& P = sim.particles;
        vec3 x4 = P[v[3]].xi;
        return mat3::from_cols(P[v[0]].xi - x4, P[v[1]].xi - x4, P[v[2]].xi - x4) * DmInv;
    }
    // gradients of C w.r.t. the 4 vertices from dC/dF
    void grads(const mat3& dCdF, vec3 g[4]) const {
        mat3 G = dCdF * DmInv.T();
        g[0] = G.col(0); g[1] = G.col(1); g[2] = G.col(2);
        g[3] = -(g[0] + g[1] + g[2]);
    }
    static mat3 cofactor(const mat3& F) {
        vec3 f1 = F.col(0), f2 = F.col(1), f3 = F.col(2);
        return mat3::from_cols(cross(f2, f3), cross(f3, f1), cross(f1, f2));
    }
    void project_positions(sim_t& sim, double dt) override {
        auto& P = sim.particles;
        double aV0 = std::fabs(V0), dt2 = dt * dt;
        double atD = 1.0 / (mu * aV0 * dt2), atH = 1.0 / (lambda * aV0 * dt2);
        mat3 F = deformation(sim);
        double cD = std::sqrt(frob2(F));
        if (!(cD > 1e-12)) return;
        double cH = F.det() - (1.0 + mu / lambda);
        vec3 gD[4], gH[4];
        grads(F * (1.0 / cD), gD);
        grads(cofactor(F), gH);
        double w[4], a11 = atD, a22 = atH, a12 = 0.0;
        for (int i = 0; i < 4; ++i) {
            w[i] = P[v[i]].invmass();
            a11 += w[i] * dot(gD[i], gD[i]);
            a22 += w[i] * dot(gH[i], gH[i]);
            a12 += w[i] * dot(gD[i], gH[i]);
        }
        double b1 = -(cD + atD * lagrange), b2 = -(cH + atH * lagrange_h);
        double det = a11 * a22 - a12 * a12;
        if (!(det > 1e-30 * a11 * a22)) return;
        double dlD = (b1 * a22 - b2 * a12) / det;
        double dlH = (b2 * a11 - b1 * a12) / det;
        lagrange += dlD;
        lagrange_h += dlH;
        for (int i = 0; i < 4; ++i) P[v[i]].xi += (gD[i] * dlD + gH[i] * dlH) * w[i];
    }
    void residual(const sim_t& sim, double dt, double& r2, double& energy) const override {
        double aV0 = std::fabs(V0), dt2 = dt * dt;
        mat3 F = deformation(sim);
        double cd = std::sqrt(frob2(F));
        double ch = F.det() - (1.0 + mu / lambda);
        double hd = cd + lagrange / (mu * aV0 * dt2);
        double hh = ch + lagrange_h / (lambda * aV0 * dt2);
        r2 += hd * hd + hh * hh;
        energy += aV0 * (0.5 * mu * (cd * cd - 3.0) + 0.5 * lambda * ch * ch);
    }
};

// ---------------------------------------------------------------------------
// distance_constraint_t: src/physics/xpbd/distance_constraint.cpp:8-53.  The
// rest length is |x0_1 - x0_2| (:20); C = |x1 - x2| - d; n = (x1 - x2)/|x1 - x2|;
// the damping term gamma * n . ((x1 - xn1) - (x2 - xn2)) as in the Green
// constraint.  One guard the reference lacks: coincident endpoints (length 0,
// where the reference divides by zero) and a zero denominator (both ends
// pinned, alpha 0) leave the constraint untouched.
struct distance_constraint_t final : constraint_t {
    uint32_t v1, v2;
    double d;
    distance_constraint_t(double a, double b, const sim_t& sim, uint32_t g1, uint32_t g2);
    void project_positions(sim_t& sim, double dt) override;
    void residual(const sim_t& sim, double dt, double& r2, double& energy) const override;
};

// ---------------------------------------------------------------------------
// collision_constraint_t: src/physics/xpbd/collision_constraint.cpp:21-48
struct collision_constraint_t final : constraint_t {
    uint32_t vi;
    vec3 q, n;
    collision_constraint_t(double a, double b, uint32_t v, vec3 p, vec3 nn)
        : constraint_t(a, b), vi(v), q(p), n(nn) {}
    double evaluate(vec3 p) const { return dot(p - q, n); }
    void project_positions(sim_t& sim, double dt) override {
        particle_t& p = sim.particles[vi];
        double w = p.invmass();
        double C = evaluate(p.xi);
        if (C >= 0.0) return;
        double at = alpha / (dt * dt);
        double dl = -(C + at * lagrange) / (w + at);
        lagrange += dl;
        p.xi += (w * n) * dl;
    }
    void residual(const sim_t& sim, double dt, double& r2, double&) const override {
        double C = evaluate(sim.particles[vi].xi);
        if (C < 0.0) { double h = C + alpha / (dt * dt) * lagrange; r2 += h * h; }
    }
};

// ---------------------------------------------------------------------------
static vec3 rotate(vec3 p, vec3 axis, double ang) {
    // Rodrigues: p cos + (k x p) sin + k (k.p)(1 - cos)
    double c = std::cos(ang), s = std::sin(ang);
    return p * c + cross(axis, p) * s + axis * (dot(axis, p) * (1.0 - c));
}

static vec3 kinematic_target(const sim_t& sim, const particle_t& p, double t) {
    const kinematic_t& k = sim.kinematics[p.kin];
    return k.center + rotate(p.x0 - k.center, k.axis, k.omega * t);
}

// Ground contacts at frame start: every surface vertex with n.x + d < 0 gets a
// collision constraint with q = x + |sd| n (bvh_model.cpp:72-94).  Plane-major
// order; vertices ascending within a plane.
static void detect_ground(sim_t& sim) {
    for (const plane_t& pl : sim.planes) {
        for (const body_t& b : sim.bodies) {
            for (uint32_t vi : b.surface) {
                vec3 p = sim.particles[vi].x;
                double sd = dot(pl.n, p) + pl.d;
                if (!(sd < 0.0)) continue;
                vec3 q = p + pl.n * std::fabs(sd);
                sim.collision_constraints.push_back(std::make_unique<collision_constraint_t>(
                    sim.prm.collision_alpha, 0.0, vi, q, pl.n));
            }
        }
        sim.ground_end.push_back((uint32_t)sim.collision_constraints.size());
    }
    // signed-distance grids: bvh_model.cpp:72-94, n = normalised gradient,
    // q = p + |sd| n
    for (const grid_t& gr : sim.grids) {
        for (const body_t& b : sim.bodies) {
            for (uint32_t vi : b.surface) {
                const vec3 p = sim.particles[vi].x;
                double sd;
                vec3 g;
                if (!gr.eval(p, sd, g) || !(sd < 0.0)) continue;
                const double l = norm(g);
                if (!(l > 0.0)) continue;
                const vec3 n = g / l;
                sim.collision_constraints.push_back(std::make_unique<collision_constraint_t>(
                    sim.prm.collision_alpha, 0.0, vi, p + n * std::fabs(sd), n));
            }
        }
        sim.ground_end.push_back((uint32_t)sim.collision_constraints.size());
    }
}

// ---------------------------------------------------------------------------
// Body-body contacts (not in the reference; its CD only meets SDFs,
// contact_handler.cpp:17).  Spatial hash: the cell of a point is
// floor(x * inv_h) per axis with x and inv_h = 1/h rounded to float and the
// product rounded to float, so CPU and GPU compute identical cells.
// Surface vertices fill the cells; every tet with at least one boundary face
// visits the cells of its AABB.  A candidate is a (surface vertex, tet) pair
// with the vertex's cell inside the tet's cell range, the vertex not a vertex
// of the tet, and the two from different bodies (or, with self contacts, from
// any body).  Narrow phase (vertex-triangle): the vertex is behind one of
// the tet's boundary triangles by less than the cell size and projects inside
// it; the contact is that triangle's half-space, frozen for the frame like
// the reference's collision constraint: q = x - d n, outward n.  One contact
// per vertex: the largest d, ties to the lower (sweep slot, face).

static inline int32_t hash_cell_coord(float x, float inv_h) { return (int32_t)std::floor(x * inv_h); }

static inline uint64_t hash_key(int32_t cx, int32_t cy, int32_t cz) {
    const uint64_t m = (1ull << 21) - 1;
    return (((uint64_t)(uint32_t)(cx + (1 << 20)) & m) << 42) | (((uint64_t)(uint32_t)(cy + (1 << 20)) & m) << 21) |
           ((uint64_t)(uint32_t)(cz + (1 << 20)) & m);
}

// Candidate (vertex, tet) pairs for float positions xf [3 * n_particles].
static void hash_candidates(const sim_t& s, const float* xf, float inv_h, int self,
                            std::vector<std::pair<uint32_t, uint32_t>>& out) {
    std::unordered_map<uint64_t, std::vector<uint32_t>> cells;
    const uint32_t n = (uint32_t)s.particles.size();
    for (uint32_t v = 0; v < n; ++v) {
        if (!s.vsurf[v]) continue;
        cells[hash_key(hash_cell_coord(xf[3 * v], inv_h), hash_cell_coord(xf[3 * v + 1], inv_h),
                       hash_cell_coord(xf[3 * v + 2], inv_h))]
            .push_back(v);
    }
    for (uint32_t t = 0; t < s.topo.size(); ++t) {
        const tet_topo_t& tt = s.topo[t];
        if (!tt.bmask) continue;
        float lo[3], hi[3];
        for (int a = 0; a < 3; ++a) {
            lo[a] = hi[a] = xf[3 * tt.v[0] + a];
            for (int k = 1; k < 4; ++k) {
                lo[a] = std::min(lo[a], xf[3 * tt.v[k] + a]);
                hi[a] = std::max(hi[a], xf[3 * tt.v[k] + a]);
            }
        }
        int32_t c0[3], c1[3];
        for (int a = 0; a < 3; ++a) {
            c0[a] = hash_cell_coord(lo[a], inv_h);
            c1[a] = hash_cell_coord(hi[a], inv_h);
        }
        for (int32_t cx = c0[0]; cx <= c1[0]; ++cx)
            for (int32_t cy = c0[1]; cy <= c1[1]; ++cy)
                for (int32_t cz = c0[2]; cz <= c1[2]; ++cz) {
                    auto it = cells.find(hash_key(cx, cy, cz));
                    if (it == cells.end()) continue;
                    for (uint32_t v : it->second) {
                        if (v == tt.v[0] || v == tt.v[1] || v == tt.v[2] || v == tt.v[3]) continue;
                        if (!self && s.vbody[v] == tt.body) continue;
                        out.push_back({v, t});
                    }
                }
    }
}

// Boundary face f of tet tt as a contact plane for point p: outward unit
// normal (oriented away from the tet's opposite vertex), signed distance d of
// p to the plane, and whether the projection of p onto the plane falls
// inside the triangle.
static bool face_plane(const sim_t& s, const tet_topo_t& tt, int f, vec3 p, double& d, vec3& n) {
    static const int F[4][4] = {{0, 1, 3, 2}, {1, 2, 3, 0}, {2, 0, 3, 1}, {0, 2, 1, 3}};  // a b c opposite
    const vec3 a = s.particles[tt.v[F[f][0]]].x, b = s.particles[tt.v[F[f][1]]].x,
               c = s.particles[tt.v[F[f][2]]].x, o = s.particles[tt.v[F[f][3]]].x;
    vec3 nn = cross(b - a, c - a);
    const double l = norm(nn);
    if (!(l > 0)) return false;
    nn = nn / l;
    if (dot(nn, o - a) > 0) nn = -nn;
    n = nn;
    d = dot(p - a, nn);
    const vec3 q = p - nn * d;
    // barycentric signs of q in (a, b, c) measured along n
    const double ua = dot(nn, cross(b - q, c - q)), ub = dot(nn, cross(c - q, a - q)),
                 uc = dot(nn, cross(a - q, b - q));
    return (ua >= 0 && ub >= 0 && uc >= 0) || (ua <= 0 && ub <= 0 && uc <= 0);
}

// Narrow phase of a candidate (vertex, tet): the vertex is behind a boundary
// triangle of the tet (-h < d < 0) and projects inside it.  One contact per
// vertex: the shallowest such triangle (largest d), ties to the lower
// (sweep slot, face).  Contact: q = x - d n, normal n (frozen for the frame).
static void detect_bodies(sim_t& sim) {
    if (!sim.prm.body_contacts || !(sim.prm.hash_cell > 0)) return;
    const float inv_h = (float)(1.0 / sim.prm.hash_cell);
    const double depth = sim.prm.hash_cell;
    const uint32_t n = (uint32_t)sim.particles.size();
    std::vector<float> xf(3 * (size_t)n);
    for (uint32_t v = 0; v < n; ++v) {
        xf[3 * v] = (float)sim.particles[v].x.x;
        xf[3 * v + 1] = (float)sim.particles[v].x.y;
        xf[3 * v + 2] = (float)sim.particles[v].x.z;
    }
    std::vector<std::pair<uint32_t, uint32_t>> cand;
    hash_candidates(sim, xf.data(), inv_h, sim.prm.body_contacts == 2, cand);
    struct best_t { double d; uint64_t key; vec3 n; };
    std::vector<best_t> best(n, best_t{-1e300, ~0ull, vec3{}});
    for (auto& c : cand) {
        const tet_topo_t& tt = sim.topo[c.second];
        const vec3 p = sim.particles[c.first].x;
        for (int f = 0; f < 4; ++f) {
            if (!((tt.bmask >> f) & 1u)) continue;
            double d; vec3 nn;
            if (!face_plane(sim, tt, f, p, d, nn)) continue;
            if (!(d < 0.0 && d > -depth)) continue;
            best_t& b = best[c.first];
            const uint64_t key = ((uint64_t)sim.slot_of_tet[c.second] << 2) | (uint64_t)f;
            if (d > b.d || (d == b.d && key < b.key)) b = best_t{d, key, nn};
        }
    }
    uint32_t nb = 0;
    for (uint32_t v = 0; v < n; ++v) {
        if (best[v].key == ~0ull) continue;
        const vec3 q = sim.particles[v].x - best[v].n * best[v].d;
        sim.collision_constraints.push_back(
            std::make_unique<collision_constraint_t>(sim.prm.collision_alpha, 0.0, v, q, best[v].n));
        ++nb;
    }
    sim.st.n_body_contacts = nb;
}

}  // namespace orc

using namespace orc;

distance_constraint_t::distance_constraint_t(double a, double b, const sim_t& sim, uint32_t g1, uint32_t g2)
    : constraint_t(a, b), v1(g1), v2(g2) {
    d = norm(sim.particles[g1].x0 - sim.particles[g2].x0);
}

void distance_constraint_t::project_positions(sim_t& sim, double dt) {
    particle_t& p1 = sim.particles[v1];
    particle_t& p2 = sim.particles[v2];
    const double w1 = p1.invmass(), w2 = p2.invmass();
    const vec3 diff = p1.xi - p2.xi;
    const double length = norm(diff);
    if (!(length > 0.0)) return;
    const vec3 n = diff / length;
    const double C = length - d;
    const double wsum = w1 + w2;
    const double dt2 = dt * dt;
    const double alpha_tilde = alpha / dt2;
    const double beta_tilde = beta * dt2;
    const double gradC_dot_disp = dot(n, p1.xi - p1.xn) - dot(n, p2.xi - p2.xn);
    const double gamma = alpha_tilde * beta_tilde / dt;
    const double num = -(C + alpha_tilde * lagrange) + gamma * gradC_dot_disp;
    const double den = (1.0 + gamma) * wsum + alpha_tilde;
    if (!(den > 0.0)) return;
    const double dl = num / den;
    lagrange += dl;
    p1.xi += n * (w1 * dl);
    p2.xi += -n * (w2 * dl);
}

void distance_constraint_t::residual(const sim_t& sim, double dt, double& r2, double& energy) const {
    const double C = norm(sim.particles[v1].xi - sim.particles[v2].xi) - d;
    const double h = C + alpha / (dt * dt) * lagrange;
    r2 += h * h;
    if (alpha > 0.0) energy += 0.5 * C * C / alpha;
}

// The elastic sweep: tets in their (colour) order, then the distance
// constraints in theirs.
static void rebuild_edge_tail(sim_t& s) {
    const size_t nt = s.constraints.size();
    s.sweep.resize(nt);
    if (s.edge_order.size() != s.edges.size()) {
        s.edge_order.resize(s.edges.size());
        for (uint32_t k = 0; k < s.edge_order.size(); ++k) s.edge_order[k] = k;
        s.edge_offsets.clear();
    }
    for (uint32_t k : s.edge_order) s.sweep.push_back(s.edges[k].get());
    if (!s.colour_offsets.empty()) {
        // tet colours first (their offsets end at nt), then the edge colours
        while (s.colour_offsets.size() > 1 && s.colour_offsets.back() > nt) s.colour_offsets.pop_back();
        if (s.edge_offsets.empty()) {
            if (!s.edges.empty()) s.colour_offsets.push_back((uint32_t)(nt + s.edges.size()));
        } else {
            for (size_t c = 1; c < s.edge_offsets.size(); ++c)
                s.colour_offsets.push_back((uint32_t)nt + s.edge_offsets[c]);
        }
    }
}

extern "C" {

void* orc_create(double alpha, double beta, double collision_alpha, const double* gravity,
                 int gravity_mode) {
    sim_t* s = new sim_t();
    s->prm.alpha = alpha;
    s->prm.beta = beta;
    s->prm.collision_alpha = collision_alpha;
    s->prm.gravity = {gravity[0], gravity[1], gravity[2]};
    s->prm.gravity_mode = gravity_mode;
    return s;
}

void orc_destroy(void* h) { delete (sim_t*)h; }

void orc_set_threads(void* h, int n) { ((sim_t*)h)->threads = n < 1 ? 1 : n; }

// Adds a body: rest shape x0 [3nv], initial positions xinit [3nv] (may be
// NULL), tets [4nt] (body-local ids).  mass [nv] (NULL -> lumped from density,
// m_v = sum density*|V0|/4).  Returns the body id.
int orc_add_body(void* h, const double* x0, const double* xinit, uint32_t nv, const uint32_t* tets,
                 uint32_t nt, int model, double E, double nu, double density, const double* mass) {
    sim_t& s = *(sim_t*)h;
    body_t b;
    b.v0 = (uint32_t)s.particles.size();
    b.nv = nv;
    b.t0 = (uint32_t)s.constraints.size();
    b.nt = nt;
    b.model = model;
    for (uint32_t i = 0; i < nv; ++i) {
        particle_t p;
        p.x0 = {x0[3 * i], x0[3 * i + 1], x0[3 * i + 2]};
        vec3 xi = xinit ? vec3{xinit[3 * i], xinit[3 * i + 1], xinit[3 * i + 2]} : p.x0;
        p.xi = p.xn = p.x = xi;
        p.m = 0.0;
        s.particles.push_back(p);
    }
    // lumped masses
    for (uint32_t t = 0; t < nt; ++t) {
        const uint32_t* q = tets + 4 * t;
        vec3 a = s.particles[b.v0 + q[0]].x0, bb = s.particles[b.v0 + q[1]].x0,
             c = s.particles[b.v0 + q[2]].x0, d = s.particles[b.v0 + q[3]].x0;
        double V = std::fabs(mat3::from_cols(a - d, bb - d, c - d).det() / 6.0);
        for (int k = 0; k < 4; ++k) s.particles[b.v0 + q[k]].m += density * V / 4.0;
    }
    if (mass)
        for (uint32_t i = 0; i < nv; ++i) s.particles[b.v0 + i].m = mass[i];
    for (uint32_t t = 0; t < nt; ++t) {
        uint32_t g[4];
        for (int k = 0; k < 4; ++k) g[k] = b.v0 + tets[4 * t + k];
        if (model == 1)
            s.constraints.push_back(std::make_unique<snh_constraint_t>(s, g, E, nu));
        else
            s.constraints.push_back(
                std::make_unique<green_constraint_t>(s.prm.alpha, s.prm.beta, s, g, E, nu));
    }
    // boundary: faces (topology.cpp:335-342) with one incident tet
    std::unordered_map<uint64_t, std::pair<int, std::array<uint32_t, 3>>> faces;
    faces.reserve(nt * 4);
    for (uint32_t t = 0; t < nt; ++t) {
        const uint32_t* q = tets + 4 * t;
        uint32_t fl[4][3] = {{q[0], q[1], q[3]}, {q[1], q[2], q[3]}, {q[2], q[0], q[3]}, {q[0], q[2], q[1]}};
        for (auto& f : fl) {
            uint32_t srt[3] = {f[0], f[1], f[2]};
            std::sort(srt, srt + 3);
            uint64_t key = ((uint64_t)srt[0] * nv + srt[1]) * (uint64_t)nv + srt[2];
            auto it = faces.find(key);
            if (it == faces.end())
                faces.emplace(key, std::make_pair(1, std::array<uint32_t, 3>{f[0], f[1], f[2]}));
            else
                it->second.first++;
        }
    }
    std::vector<uint32_t> surf;
    for (auto& kv : faces) {
        if (kv.second.first == 2) continue;
        for (int k = 0; k < 3; ++k) surf.push_back(b.v0 + kv.second.second[k]);
        if (kv.second.first == 1)
            b.surface_tris.push_back({b.v0 + kv.second.second[0], b.v0 + kv.second.second[1],
                                      b.v0 + kv.second.second[2]});
    }
    std::sort(surf.begin(), surf.end());
    surf.erase(std::unique(surf.begin(), surf.end()), surf.end());
    std::sort(b.surface_tris.begin(), b.surface_tris.end());
    // visual model (tetrahedral_mesh_boundary.cpp:76-120): the tet mesh lists
    // each distinct face once, at its first appearance over the tets in order
    // and their faces_copy faces (topology.cpp:335-342, add_tetrahedron
    // :904-950), keeping that appearance's winding; faces with != 2 incident
    // tets are boundary triangles; surface vertices are numbered by first
    // appearance in them
    {
        std::unordered_map<uint64_t, uint8_t> seen;
        std::unordered_map<uint32_t, uint32_t> local;
        for (uint32_t t = 0; t < nt; ++t) {
            const uint32_t* q = tets + 4 * t;
            const uint32_t fl[4][3] = {{q[0], q[1], q[3]}, {q[1], q[2], q[3]}, {q[2], q[0], q[3]}, {q[0], q[2], q[1]}};
            for (auto& f : fl) {
                uint32_t srt[3] = {f[0], f[1], f[2]};
                std::sort(srt, srt + 3);
                const uint64_t key = ((uint64_t)srt[0] * nv + srt[1]) * (uint64_t)nv + srt[2];
                if (faces[key].first == 2 || !seen.emplace(key, 1).second) continue;
                std::array<uint32_t, 3> tri;
                for (int j = 0; j < 3; ++j) {
                    auto it = local.find(f[j]);
                    if (it == local.end()) {
                        it = local.emplace(f[j], (uint32_t)b.vis_map.size()).first;
                        b.vis_map.push_back(b.v0 + f[j]);
                    }
                    tri[j] = it->second;
                }
                b.vis_tris.push_back(tri);
            }
        }
        b.vis_normal.assign(b.vis_map.size(), vec3{0.0, 0.0, 0.0});
        update_visual_model(s.particles, b, nullptr);   // tetrahedral_body.cpp:25
    }
    // per-tet boundary faces and body ids for the spatial hash
    const uint32_t body_id = (uint32_t)s.bodies.size();
    s.vbody.resize(s.particles.size(), body_id);
    s.vsurf.resize(s.particles.size(), 0);
    for (uint32_t v : surf) s.vsurf[v] = 1;
    for (uint32_t t = 0; t < nt; ++t) {
        const uint32_t* q = tets + 4 * t;
        const uint32_t fl[4][3] = {{q[0], q[1], q[3]}, {q[1], q[2], q[3]}, {q[2], q[0], q[3]}, {q[0], q[2], q[1]}};
        tet_topo_t tt;
        for (int k = 0; k < 4; ++k) tt.v[k] = b.v0 + q[k];
        tt.body = body_id;
        tt.bmask = 0;
        for (int f = 0; f < 4; ++f) {
            uint32_t srt[3] = {fl[f][0], fl[f][1], fl[f][2]};
            std::sort(srt, srt + 3);
            uint64_t key = ((uint64_t)srt[0] * nv + srt[1]) * (uint64_t)nv + srt[2];
            if (faces[key].first == 1) tt.bmask |= (uint8_t)(1u << f);
        }
        s.topo.push_back(tt);
    }
    b.surface = std::move(surf);
    s.bodies.push_back(std::move(b));
    s.sweep.clear();
    for (auto& c : s.constraints) s.sweep.push_back(c.get());
    s.slot_of_tet.resize(s.constraints.size());
    for (uint32_t k = 0; k < s.slot_of_tet.size(); ++k) s.slot_of_tet[k] = k;
    s.colour_offsets.clear();
    rebuild_edge_tail(s);
    return (int)s.bodies.size() - 1;
}

void orc_pin(void* h, int body, const uint32_t* v, uint32_t n) {
    sim_t& s = *(sim_t*)h;
    for (uint32_t i = 0; i < n; ++i) s.particles[s.bodies[body].v0 + v[i]].m = 0.0;
}

void orc_add_kinematic_rotation(void* h, int body, const uint32_t* v, uint32_t n, const double* c,
                                const double* axis, double omega) {
    sim_t& s = *(sim_t*)h;
    kinematic_t k;
    k.center = {c[0], c[1], c[2]};
    vec3 a{axis[0], axis[1], axis[2]};
    k.axis = a / norm(a);
    k.omega = omega;
    s.kinematics.push_back(k);
    for (uint32_t i = 0; i < n; ++i) {
        particle_t& p = s.particles[s.bodies[body].v0 + v[i]];
        p.m = 0.0;
        p.kin = (int)s.kinematics.size() - 1;
    }
}

void orc_set_external_acceleration(void* h, int body, const double* acc) {
    sim_t& s = *(sim_t*)h;
    const body_t& b = s.bodies[body];
    for (uint32_t i = 0; i < b.nv; ++i)
        s.particles[b.v0 + i].ext_acc = {acc[3 * i], acc[3 * i + 1], acc[3 * i + 2]};
}

void orc_add_sdf_grid(void* h, const float* values, const uint32_t* nodes, const double* origin,
                      const double* spacing) {
    sim_t& s = *(sim_t*)h;
    grid_t g;
    size_t n = 1;
    for (int k = 0; k < 3; ++k) {
        g.n[k] = nodes[k];
        g.o[k] = origin[k];
        g.h[k] = spacing[k];
        n *= nodes[k];
    }
    g.v.assign(values, values + n);
    s.grids.push_back(std::move(g));
}

// A cubic grid (layout of grid_t) of cells[3] cells.
void orc_add_sdf_grid_cubic(void* h, const float* values, const uint32_t* cells, const double* origin,
                            const double* spacing) {
    sim_t& s = *(sim_t*)h;
    grid_t g;
    g.cubic = true;
    for (int k = 0; k < 3; ++k) {
        g.n[k] = cells[k] + 1;
        g.o[k] = origin[k];
        g.h[k] = spacing[k];
    }
    const size_t nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const size_t n = nx * ny * nz + 2 * ((nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1));
    g.v.assign(values, values + n);
    s.grids.push_back(std::move(g));
}

// The cubic cell interpolant alone (for its tests): value and gradient of
// grid `gi` at p; returns 0 outside the grid.
int orc_grid_eval(void* h, int gi, const double* p, double* out4) {
    const grid_t& g = ((sim_t*)h)->grids[gi];
    double sd;
    vec3 gr;
    if (!g.eval(vec3{p[0], p[1], p[2]}, sd, gr)) return 0;
    out4[0] = sd;
    out4[1] = gr.x;
    out4[2] = gr.y;
    out4[3] = gr.z;
    return 1;
}

void orc_add_ground_plane(void* h, const double* n, double d) {
    sim_t& s = *(sim_t*)h;
    vec3 nn{n[0], n[1], n[2]};
    double l = norm(nn);
    s.planes.push_back({nn / l, d / l});
}

// Permute the elastic constraint list: order[k] = global tet id projected k-th.
// offsets (n_colours+1 entries, may be NULL) mark vertex-disjoint groups that
// may run in parallel when threads > 1.
int orc_set_tet_order(void* h, const uint32_t* order, uint32_t n, const uint32_t* offsets,
                      uint32_t n_colours) {
    sim_t& s = *(sim_t*)h;
    if (n != s.constraints.size()) return 1;
    s.sweep.resize(n);
    for (uint32_t k = 0; k < n; ++k) {
        if (order[k] >= n) return 1;
        s.sweep[k] = s.constraints[order[k]].get();
        s.slot_of_tet[order[k]] = k;
    }
    s.colour_offsets.clear();
    if (offsets) s.colour_offsets.assign(offsets, offsets + n_colours + 1);
    rebuild_edge_tail(s);
    return 0;
}

// The oracle's own colour-parallel plan, independent of the CUDA library:
// first-fit colouring of the tets in list order (each tet takes the lowest
// colour none of its four vertices has yet), then the list colour-major with
// list order kept inside a colour.  Tets of one colour share no vertex, so a
// colour's projections commute and the colour-parallel sweep over this order
// equals the sequential sweep over it.  Writes order [n_tets] and offsets
// [n_colours + 1] (cap_offsets entries available); returns n_colours, or 0
// when cap_offsets is too small.
uint32_t orc_plan_colours(void* h, uint32_t* order, uint32_t* offsets, uint32_t cap_offsets) {
    sim_t& s = *(sim_t*)h;
    const size_t nt = s.topo.size();
    std::vector<std::vector<uint64_t>> used(s.particles.size());   // per vertex: colour bit words
    std::vector<uint32_t> colour(nt);
    uint32_t n_colours = 0;
    for (size_t t = 0; t < nt; ++t) {
        const uint32_t* v = s.topo[t].v;
        uint32_t c = 0;
        for (;; ++c) {
            const size_t w = c >> 6;
            const uint64_t bit = 1ull << (c & 63);
            bool taken = false;
            for (int k = 0; k < 4 && !taken; ++k) taken = w < used[v[k]].size() && (used[v[k]][w] & bit);
            if (!taken) break;
        }
        colour[t] = c;
        for (int k = 0; k < 4; ++k) {
            auto& u = used[v[k]];
            if (u.size() <= (c >> 6)) u.resize((c >> 6) + 1, 0);
            u[c >> 6] |= 1ull << (c & 63);
        }
        n_colours = std::max(n_colours, c + 1);
    }
    if (cap_offsets < n_colours + 1) return 0;
    std::vector<uint32_t> count(n_colours + 1, 0);
    for (size_t t = 0; t < nt; ++t) ++count[colour[t] + 1];
    for (uint32_t c = 0; c < n_colours; ++c) count[c + 1] += count[c];
    for (uint32_t c = 0; c <= n_colours; ++c) offsets[c] = count[c];
    for (size_t t = 0; t < nt; ++t) order[count[colour[t]]++] = (uint32_t)t;
    return n_colours;
}

// distance_constraint_t objects (distance_constraint.cpp:8-22) for n 4-tuples
// (b1, b2, v1, v2), as the reference's constructor takes them.
int orc_add_distance(void* h, const uint32_t* ids, uint32_t n, double alpha, double beta) {
    sim_t& s = *(sim_t*)h;
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t b1 = ids[4 * k], b2 = ids[4 * k + 1], v1 = ids[4 * k + 2], v2 = ids[4 * k + 3];
        if (b1 >= s.bodies.size() || b2 >= s.bodies.size() || v1 >= s.bodies[b1].nv || v2 >= s.bodies[b2].nv)
            return 1;
        s.edges.push_back(std::make_unique<distance_constraint_t>(alpha, beta, s, s.bodies[b1].v0 + v1,
                                                                  s.bodies[b2].v0 + v2));
    }
    s.edge_order.clear();
    rebuild_edge_tail(s);
    return 0;
}

// Projection order of the distance constraints (input indices, colour-major)
// with n_colours + 1 colour offsets (may be NULL).
int orc_set_edge_order(void* h, const uint32_t* order, uint32_t n, const uint32_t* offsets, uint32_t n_colours) {
    sim_t& s = *(sim_t*)h;
    if (n != s.edges.size()) return 1;
    for (uint32_t k = 0; k < n; ++k)
        if (order[k] >= n) return 1;
    s.edge_order.assign(order, order + n);
    s.edge_offsets.clear();
    if (offsets) s.edge_offsets.assign(offsets, offsets + n_colours + 1);
    rebuild_edge_tail(s);
    return 0;
}

void orc_get_distance_lambdas(void* h, double* out) {
    sim_t& s = *(sim_t*)h;
    for (size_t k = 0; k < s.edges.size(); ++k) out[k] = s.edges[k]->lagrange;
}

static void compute_residual(sim_t& s, double dt, double& r2e, double& r2c, double& energy) {
    r2e = r2c = energy = 0;
    for (auto* c : s.sweep) c->residual(s, dt, r2e, energy);
    double dummy = 0;
    for (auto& c : s.collision_constraints) c->residual(s, dt, r2c, dummy);
}

static void project_sweep(sim_t& s, double dt) {
    const size_t n = s.sweep.size();
#ifdef _OPENMP
    if (s.threads > 1 && !s.colour_offsets.empty()) {
        for (size_t c = 0; c + 1 < s.colour_offsets.size(); ++c) {
            int64_t b = s.colour_offsets[c], e = s.colour_offsets[c + 1];
            if (e - b < 256) {
                for (int64_t k = b; k < e; ++k) s.sweep[k]->project_positions(s, dt);
            } else {
#pragma omp parallel for num_threads(s.threads) schedule(static)
                for (int64_t k = b; k < e; ++k) s.sweep[k]->project_positions(s, dt);
            }
        }
        return;
    }
#endif
    for (size_t k = 0; k < n; ++k) s.sweep[k]->project_positions(s, dt);
}

// gauss_seidel_solver_t::solve (gauss_seidel_solver.cpp:8-37): reset every
// multiplier, then per iteration all collision constraints, then all elastic
// constraints, in list order.
void orc_solve(void* h, double dt, uint32_t iterations) {
    sim_t& s = *(sim_t*)h;
    for (auto& c : s.collision_constraints) c->prepare_for_projection();
    for (auto* c : s.sweep) c->prepare_for_projection();
    s.residual_history.clear();
    for (uint32_t k = 0; k < iterations; ++k) {
        for (auto& c : s.collision_constraints) c->project_positions(s, dt);
        project_sweep(s, dt);
        s.st.projections += s.constraints.size();
        if (s.record_history) {
            double r2e, r2c, e;
            compute_residual(s, dt, r2e, r2c, e);
            s.residual_history.push_back(std::sqrt(r2e + r2c));
        }
    }
}

static void predict(sim_t& s, double dt) {
    const double t_next = s.time + dt;
    const int64_t n = (int64_t)s.particles.size();
#pragma omp parallel for num_threads(s.threads) schedule(static) if (s.threads > 1)
    for (int64_t i = 0; i < n; ++i) {
        particle_t& p = s.particles[i];
        if (p.kin >= 0) {
            p.xi = kinematic_target(s, p, t_next);
            continue;
        }
        // timestep.cpp:39-41 applies gravity as a force of -9.81 on y; the
        // acceleration mode applies m*g so that a = g for any mass.
        if (s.prm.gravity_mode == 1) p.f += s.prm.gravity;
        else p.f += s.prm.gravity * p.m;
        p.f += p.ext_acc * p.m;
        p.v = p.v + p.a() * dt;
        p.xi = p.x + p.v * dt;
    }
}

static void finalize(sim_t& s, double dt) {
    const int64_t n = (int64_t)s.particles.size();
#pragma omp parallel for num_threads(s.threads) schedule(static) if (s.threads > 1)
    for (int64_t i = 0; i < n; ++i) {
        particle_t& p = s.particles[i];
        p.x = p.xi;                  // timestep.cpp:52-55
        p.v = (p.x - p.xn) / dt;
        p.xn = p.x;
        p.f = {0, 0, 0};
    }
}

void orc_detect_contacts(void* h) {
    sim_t& s = *(sim_t*)h;
    s.collision_constraints.clear();
    s.ground_end.clear();
    detect_ground(s);
    s.st.n_contacts = (uint32_t)s.collision_constraints.size();
    s.st.n_body_contacts = 0;
    detect_bodies(s);   // after the ground contacts: collision list = [ground..., bodies...]
}

// mode 0 off, 1 between bodies, 2 also within a body; cell size h (metres).
void orc_set_body_contacts(void* h, int mode, double cell) {
    sim_t& s = *(sim_t*)h;
    s.prm.body_contacts = mode;
    s.prm.hash_cell = cell;
}

// Candidate (vertex, tet) pairs of the spatial hash for float positions
// xf [3 * n] (add order), sorted as (vertex << 32 | tet).  Returns the count.
uint64_t orc_hash_candidates(void* h, const float* xf, double cell, int self, uint64_t* out, uint64_t cap) {
    sim_t& s = *(sim_t*)h;
    std::vector<std::pair<uint32_t, uint32_t>> c;
    hash_candidates(s, xf, (float)(1.0 / cell), self, c);
    std::vector<uint64_t> k(c.size());
    for (size_t i = 0; i < c.size(); ++i) k[i] = ((uint64_t)c[i].first << 32) | c[i].second;
    std::sort(k.begin(), k.end());
    for (size_t i = 0; i < k.size() && i < cap; ++i) out[i] = k[i];
    return k.size();
}

uint32_t orc_n_body_contacts(void* h) { return ((sim_t*)h)->st.n_body_contacts; }

// timestep_t::step (timestep.cpp:20-70): contacts once per frame from x, then
// per substep predict -> solve -> set x, v.
void orc_step(void* h, double frame_dt, uint32_t substeps, uint32_t iterations) {
    sim_t& s = *(sim_t*)h;
    double dt = frame_dt / (double)substeps;
    orc_detect_contacts(h);
    for (uint32_t k = 0; k < substeps; ++k) {
        predict(s, dt);
        orc_solve(h, dt, iterations);
        double r2e, r2c, e;
        compute_residual(s, dt, r2e, r2c, e);
        s.st.r2_elastic = r2e;
        s.st.r2_contact = r2c;
        s.st.residual = std::sqrt(r2e + r2c);
        s.st.energy = e;
        finalize(s, dt);
        s.time += dt;
    }
    s.collision_constraints.clear();   // timestep.cpp:68
}

// Same as orc_step but without the residual pass (timing path).
void orc_step_fast(void* h, double frame_dt, uint32_t substeps, uint32_t iterations) {
    sim_t& s = *(sim_t*)h;
    double dt = frame_dt / (double)substeps;
    orc_detect_contacts(h);
    for (uint32_t k = 0; k < substeps; ++k) {
        predict(s, dt);
        orc_solve(h, dt, iterations);
        finalize(s, dt);
        s.time += dt;
    }
    s.collision_constraints.clear();
}

void orc_predict(void* h, double dt) { predict(*(sim_t*)h, dt); }
void orc_finalize(void* h, double dt) { sim_t& s = *(sim_t*)h; finalize(s, dt); s.time += dt; }

void orc_residual(void* h, double dt, double* out3) {
    sim_t& s = *(sim_t*)h;
    double r2e, r2c, e;
    compute_residual(s, dt, r2e, r2c, e);
    out3[0] = std::sqrt(r2e + r2c);
    out3[1] = e;
    out3[2] = std::sqrt(r2e);
}

void orc_set_record_history(void* h, int on) { ((sim_t*)h)->record_history = on; }
uint32_t orc_get_history(void* h, double* out, uint32_t cap) {
    sim_t& s = *(sim_t*)h;
    uint32_t n = (uint32_t)std::min<size_t>(cap, s.residual_history.size());
    for (uint32_t i = 0; i < n; ++i) out[i] = s.residual_history[i];
    return (uint32_t)s.residual_history.size();
}

// field: 0 x, 1 xi, 2 v, 3 x0
void orc_get(void* h, int field, double* out) {
    sim_t& s = *(sim_t*)h;
    for (size_t i = 0; i < s.particles.size(); ++i) {
        const particle_t& p = s.particles[i];
        vec3 q = field == 0 ? p.x : field == 1 ? p.xi : field == 2 ? p.v : p.x0;
        out[3 * i] = q.x; out[3 * i + 1] = q.y; out[3 * i + 2] = q.z;
    }
}

void orc_set(void* h, int field, const double* in) {
    sim_t& s = *(sim_t*)h;
    for (size_t i = 0; i < s.particles.size(); ++i) {
        particle_t& p = s.particles[i];
        vec3 q{in[3 * i], in[3 * i + 1], in[3 * i + 2]};
        if (field == 0) { p.x = q; p.xn = q; p.xi = q; }
        else if (field == 1) p.xi = q;
        else if (field == 2) p.v = q;
    }
}

void orc_get_masses(void* h, double* out) {
    sim_t& s = *(sim_t*)h;
    for (size_t i = 0; i < s.particles.size(); ++i) out[i] = s.particles[i].m;
}

uint32_t orc_get_surface(void* h, int body, uint32_t* out, uint32_t cap) {
    sim_t& s = *(sim_t*)h;
    const auto& v = s.bodies[body].surface;
    for (uint32_t i = 0; i < v.size() && i < cap; ++i) out[i] = v[i];
    return (uint32_t)v.size();
}

// Lagrange multipliers in global tet order (2 per tet: deviatoric/StVK, hydrostatic).
void orc_get_lambdas(void* h, double* out) {
    sim_t& s = *(sim_t*)h;
    for (size_t i = 0; i < s.constraints.size(); ++i) {
        out[2 * i] = s.constraints[i]->lagrange;
        auto* sn = dynamic_cast<snh_constraint_t*>(s.constraints[i].get());
        out[2 * i + 1] = sn ? sn->lagrange_h : 0.0;
    }
}

// Contacts of the current frame (after orc_detect_contacts): vertex, q, n.
uint32_t orc_get_contacts(void* h, uint32_t* verts, double* qn, uint32_t cap) {
    sim_t& s = *(sim_t*)h;
    uint32_t n = 0;
    for (auto& c : s.collision_constraints) {
        auto* cc = dynamic_cast<collision_constraint_t*>(c.get());
        if (!cc) continue;
        if (n < cap) {
            verts[n] = cc->vi;
            qn[6 * n + 0] = cc->q.x; qn[6 * n + 1] = cc->q.y; qn[6 * n + 2] = cc->q.z;
            qn[6 * n + 3] = cc->n.x; qn[6 * n + 4] = cc->n.y; qn[6 * n + 5] = cc->n.z;
        }
        ++n;
    }
    return n;
}

// Single-constraint probes (unit tests): evaluate psi and f_i for one tet.
void orc_tet_eval(void* h, uint32_t tet, double* psi, double* f12) {
    sim_t& s = *(sim_t*)h;
    auto* g = dynamic_cast<green_constraint_t*>(s.constraints[tet].get());
    if (!g) { *psi = NAN; return; }
    vec3 f[4];
    g->evaluate(s, *psi, f);
    for (int i = 0; i < 4; ++i) { f12[3 * i] = f[i].x; f12[3 * i + 1] = f[i].y; f12[3 * i + 2] = f[i].z; }
}

void orc_svd3(const double* F9, double* U9, double* s3, double* V9) {
    mat3 F, U, V; vec3 s;
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) F.m[i][j] = F9[3 * i + j];
    svd3(F, U, s, V);
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) { U9[3 * i + j] = U.m[i][j]; V9[3 * i + j] = V.m[i][j]; }
    s3[0] = s.x; s3[1] = s.y; s3[2] = s.z;
}

// Visual model of a body: triangles (surface-local ids) and surface vertex ->
// body-local vertex map; returns counts through n_tri / n_sv.
void orc_surface_mesh(void* h, int body, uint32_t* tris, uint32_t cap_tri, uint32_t* n_tri, uint32_t* vmap,
                      uint32_t cap_sv, uint32_t* n_sv) {
    const body_t& b = ((sim_t*)h)->bodies[body];
    *n_tri = (uint32_t)b.vis_tris.size();
    *n_sv = (uint32_t)b.vis_map.size();
    for (uint32_t i = 0; i < b.vis_tris.size() && i < cap_tri; ++i)
        for (int j = 0; j < 3; ++j) tris[3 * i + j] = b.vis_tris[i][j];
    for (uint32_t i = 0; i < b.vis_map.size() && i < cap_sv; ++i) vmap[i] = b.vis_map[i] - b.v0;
}

// One visual-model update (accumulate = 0 clears the normals first, which the
// reference never does); pos / nrm receive [3 * n_sv] each.
void orc_update_surface(void* h, int body, int accumulate, double* pos, double* nrm) {
    sim_t& s = *(sim_t*)h;
    body_t& b = s.bodies[body];
    if (!accumulate) b.vis_normal.assign(b.vis_map.size(), vec3{0.0, 0.0, 0.0});
    std::vector<vec3> p;
    update_visual_model(s.particles, b, &p);
    for (size_t i = 0; i < p.size(); ++i) {
        pos[3 * i] = p[i].x; pos[3 * i + 1] = p[i].y; pos[3 * i + 2] = p[i].z;
        nrm[3 * i] = b.vis_normal[i].x; nrm[3 * i + 1] = b.vis_normal[i].y; nrm[3 * i + 2] = b.vis_normal[i].z;
    }
}

double orc_time(void* h) { return ((sim_t*)h)->time; }
uint64_t orc_projections(void* h) { return ((sim_t*)h)->st.projections; }
uint32_t orc_n_contacts(void* h) { return ((sim_t*)h)->st.n_contacts; }
void orc_stats(void* h, double* out4) {
    sim_t& s = *(sim_t*)h;
    out4[0] = s.st.residual; out4[1] = s.st.energy;
    out4[2] = std::sqrt(s.st.r2_elastic); out4[3] = std::sqrt(s.st.r2_contact);
}

// Wall-clock of n frames (steady_clock, as the reference's throttler times a
// step: src/rendering/physics_timestep_throttler.cpp:36-43).
double orc_time_frames(void* h, double frame_dt, uint32_t substeps, uint32_t iterations, uint32_t n) {
    auto t0 = std::chrono::steady_clock::now();
    for (uint32_t i = 0; i < n; ++i) orc_step_fast(h, frame_dt, substeps, iterations);
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
