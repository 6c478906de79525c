// sbs_gpu_timestep.hpp - header-only C++ drop-in for sbs::physics::timestep_t.
//
// Mirrors the interface of timestep_t (include/sbs/physics/timestep.h:14-33):
// dt(), iterations(), substeps() accessors and step(simulation).  step() runs
// the whole frame on the GPU through the C ABI of sbs_gpu.h instead of
// timestep.cpp:20-70 + gauss_seidel_solver.cpp:8-37, and copies positions and
// velocities back into the host particles so the caller's unchanged
// visual-model code (body->update_visual_model(), timestep.cpp:60-66) keeps
// working.
//
// `Simulation` is any type shaped like sbs::physics::simulation_t:
//   sim.particles()            -> std::vector<std::vector<Particle>> (one per body)
//   p.x0(), p.x(), p.v()       -> 3-vectors with operator()(i) or [i]
//   p.mass()                   -> mass (0 pins the particle, particle.cpp:45-49)
// and `Tets(sim, body)` returns the body's tets as 4 indices each (for the
// reference: the body's tetrahedron_set_t, tetrahedral_body.cpp:40-51).
//
// Usage in the reference's main.cpp (one line changes, :120-130):
//     sbs::gpu::gpu_timestep_t timestep{};            // was sbs::physics::timestep_t
//     timestep.dt() = 0.016; timestep.iterations() = 5u; timestep.substeps() = 1u;
//     ... throttler lambda calls timestep.step(simulation) as before.
#ifndef SBS_GPU_TIMESTEP_HPP
#define SBS_GPU_TIMESTEP_HPP

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "sbs_gpu.h"

namespace sbs {
namespace gpu {

class error : public std::runtime_error {
  public:
    error(sbs_status s, const std::string& what) : std::runtime_error(what), status(s) {}
    sbs_status status;
};

inline void check(sbs_status s, const sbs_gpu* h = nullptr) {
    if (s != SBS_OK) throw error(s, std::string(sbs_gpu_status_string(s)) + ": " + sbs_gpu_last_error(h));
}

template <typename V>
inline double comp(const V& v, int i) {
    return static_cast<double>(v[i]);
}

struct body_material {
    sbs_model model = SBS_MODEL_STVK;
    double young = 1e6;    // simulation_parameters.h:18
    double poisson = 0.3;  // simulation_parameters.h:19
    double density = 1000.0;
};

// Frame stepper with the interface of timestep_t.
class gpu_timestep_t {
  public:
    gpu_timestep_t() { sbs_gpu_params_default(&params_); }
    gpu_timestep_t(double dt, std::size_t iterations, std::size_t substeps) : gpu_timestep_t() {
        dt_ = dt;
        iterations_ = iterations;
        substeps_ = substeps;
    }
    gpu_timestep_t(const gpu_timestep_t&) = delete;
    gpu_timestep_t& operator=(const gpu_timestep_t&) = delete;
    ~gpu_timestep_t() {
        if (h_) sbs_gpu_destroy(h_);
    }

    double dt() const { return dt_; }
    double& dt() { return dt_; }
    std::size_t iterations() const { return iterations_; }
    std::size_t& iterations() { return iterations_; }
    std::size_t substeps() const { return substeps_; }
    std::size_t& substeps() { return substeps_; }
    sbs_gpu_params& params() { return params_; }

    // Scene description, given once before the first step (the reference
    // builds the same information into its constraint list, main.cpp:37-72).
    void set_material(std::size_t body, body_material m) {
        if (materials_.size() <= body) materials_.resize(body + 1);
        materials_[body] = m;
    }
    void set_tets(std::size_t body, std::vector<uint32_t> tets) {
        if (tets_.size() <= body) tets_.resize(body + 1);
        tets_[body] = std::move(tets);
    }
    void add_ground_plane(const double n[3], double d) { planes_.push_back({n[0], n[1], n[2], d}); }

    // timestep_t::step (timestep.cpp:20-70) on the GPU.
    template <typename Simulation>
    void step(Simulation& sim) {
        auto& parts = sim.particles();
        if (!h_) build(parts);
        // upload host state (the host may have changed it between frames)
        for (std::size_t b = 0; b < parts.size(); ++b) {
            const auto& ps = parts[b];
            xs_.resize(3 * ps.size());
            vs_.resize(3 * ps.size());
            for (std::size_t i = 0; i < ps.size(); ++i)
                for (int k = 0; k < 3; ++k) {
                    xs_[3 * i + k] = static_cast<float>(comp(ps[i].x(), k));
                    vs_[3 * i + k] = static_cast<float>(comp(ps[i].v(), k));
                }
            check(sbs_gpu_set_state(h_, static_cast<int32_t>(b), xs_.data(), vs_.data()), h_);
        }
        check(sbs_gpu_step(h_, dt_, static_cast<uint32_t>(substeps_), static_cast<uint32_t>(iterations_)), h_);
        for (std::size_t b = 0; b < parts.size(); ++b) {
            auto& ps = parts[b];
            xs_.resize(3 * ps.size());
            vs_.resize(3 * ps.size());
            check(sbs_gpu_get_state(h_, static_cast<int32_t>(b), xs_.data(), vs_.data()), h_);
            for (std::size_t i = 0; i < ps.size(); ++i)
                for (int k = 0; k < 3; ++k) {
                    ps[i].x()[k] = xs_[3 * i + k];
                    ps[i].xi()[k] = xs_[3 * i + k];
                    ps[i].xn()[k] = xs_[3 * i + k];
                    ps[i].v()[k] = vs_[3 * i + k];
                }
        }
    }

    sbs_gpu* handle() { return h_; }

  private:
    template <typename Parts>
    void build(Parts& parts) {
        check(sbs_gpu_create(&params_, &h_));
        for (std::size_t b = 0; b < parts.size(); ++b) {
            const auto& ps = parts[b];
            if (b >= tets_.size() || tets_[b].empty()) throw error(SBS_EINVAL, "gpu_timestep_t: body without tets");
            std::vector<double> x0(3 * ps.size()), x(3 * ps.size()), m(ps.size());
            for (std::size_t i = 0; i < ps.size(); ++i) {
                for (int k = 0; k < 3; ++k) {
                    x0[3 * i + k] = comp(ps[i].x0(), k);
                    x[3 * i + k] = comp(ps[i].x(), k);
                }
                m[i] = static_cast<double>(ps[i].mass());
            }
            body_material mat = b < materials_.size() ? materials_[b] : body_material{};
            sbs_gpu_material gm{mat.model, mat.young, mat.poisson, mat.density};
            int32_t id = 0;
            // per-particle masses are taken from the host particles (the
            // reference's particle_t::mass(), mass 0 pins)
            check(sbs_gpu_add_body(h_, x0.data(), x.data(), static_cast<uint32_t>(ps.size()), tets_[b].data(),
                                   static_cast<uint32_t>(tets_[b].size() / 4), &gm, m.data(), &id),
                  h_);
        }
        for (const auto& p : planes_) {
            const double n[3] = {p[0], p[1], p[2]};
            check(sbs_gpu_add_ground_plane(h_, n, p[3]), h_);
        }
        check(sbs_gpu_finalize(h_), h_);
    }

    sbs_gpu_params params_{};
    sbs_gpu* h_ = nullptr;
    double dt_ = 0.0;
    std::size_t iterations_ = 0, substeps_ = 0;
    std::vector<body_material> materials_;
    std::vector<std::vector<uint32_t>> tets_;
    std::vector<std::vector<double>> planes_;
    std::vector<float> xs_, vs_;
};

}  // namespace gpu
}  // namespace sbs

#endif  // SBS_GPU_TIMESTEP_HPP
