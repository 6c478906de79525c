// Drives the header-only gpu_timestep_t adapter the way the reference's
// main.cpp drives timestep_t (main.cpp:120-130): host-owned particles in
// per-body vectors, a step per frame, positions read back into the particles.
// The particle and simulation types below have the shape of
// sbs::physics::particle_t / simulation_t (particle.h:10-53, simulation.h:20-48).
//
// Scene: a 4x2x2-vertex bar (reference vertex indexing and 5-tet split,
// get_simple_bar_model.cpp), x = 0 face pinned through mass 0, ground y = -1.
// Prints the final positions, one vertex per line, for comparison.
#include <array>
#include <cstdlib>
#include <cstdio>
#include <vector>

#include "sbs_gpu_timestep.hpp"

struct vec3 {
    double v[3] = {0, 0, 0};
    double& operator[](int i) { return v[i]; }
    double operator[](int i) const { return v[i]; }
};

struct particle_t {
    vec3 x0_, x_, xi_, xn_, v_;
    double m_ = 1.0;
    vec3& x0() { return x0_; }
    vec3& x() { return x_; }
    vec3& xi() { return xi_; }
    vec3& xn() { return xn_; }
    vec3& v() { return v_; }
    const vec3& x0() const { return x0_; }
    const vec3& x() const { return x_; }
    const vec3& v() const { return v_; }
    double mass() const { return m_; }
};

struct simulation_t {
    std::vector<std::vector<particle_t>> parts;
    std::vector<std::vector<particle_t>>& particles() { return parts; }
};

int main(int argc, char** argv) {
    const int frames = argc > 1 ? std::atoi(argv[1]) : 30;
    const int W = 4, H = 2, D = 2;
    simulation_t sim;
    sim.parts.resize(1);
    for (int i = 0; i < W; ++i)
        for (int j = 0; j < H; ++j)
            for (int k = 0; k < D; ++k) {
                particle_t p;
                p.x0_ = {{0.1 * i, 0.1 * j, 0.1 * k}};
                p.x_ = p.xi_ = p.xn_ = p.x0_;
                p.m_ = i == 0 ? 0.0 : 0.25;
                sim.parts[0].push_back(p);
            }
    std::vector<uint32_t> tets;
    auto id = [&](int i, int j, int k) { return (uint32_t)(i * H * D + j * D + k); };
    for (int i = 0; i + 1 < W; ++i)
        for (int j = 0; j + 1 < H; ++j)
            for (int k = 0; k + 1 < D; ++k) {
                uint32_t p0 = id(i, j, k), p1 = id(i + 1, j, k), p2 = id(i + 1, j + 1, k), p3 = id(i, j + 1, k);
                uint32_t p4 = id(i, j, k + 1), p5 = id(i + 1, j, k + 1), p6 = id(i + 1, j + 1, k + 1),
                         p7 = id(i, j + 1, k + 1);
                std::array<std::array<uint32_t, 4>, 5> t;
                if ((i + j + k) % 2 == 1)
                    t = {{{p1, p0, p5, p2}, {p5, p2, p7, p6}, {p7, p0, p5, p4}, {p2, p0, p7, p3}, {p5, p0, p7, p2}}};
                else
                    t = {{{p3, p1, p4, p0}, {p6, p1, p3, p2}, {p4, p1, p6, p5}, {p6, p3, p4, p7}, {p3, p1, p6, p4}}};
                for (auto& q : t) tets.insert(tets.end(), q.begin(), q.end());
            }
    sbs::gpu::gpu_timestep_t timestep{};
    timestep.dt() = 1.0 / 60.0;
    timestep.iterations() = 10u;
    timestep.substeps() = 1u;
    timestep.set_tets(0, tets);
    timestep.set_material(0, {SBS_MODEL_STVK, 1e5, 0.3, 1000.0});
    const double n[3] = {0.0, 1.0, 0.0};
    timestep.add_ground_plane(n, 1.0);
    try {
        for (int f = 0; f < frames; ++f) timestep.step(sim);
    } catch (const sbs::gpu::error& e) {
        std::fprintf(stderr, "adapter error: %s\n", e.what());
        return 2;
    }
    for (const auto& p : sim.parts[0]) std::printf("%.9g %.9g %.9g\n", p.x_[0], p.x_[1], p.x_[2]);
    return 0;
}
