// Internal device-side layout of one scene and the kernel entry points.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sdf_eval.cuh"

namespace sbs {

constexpr int kMaxColours = 128;  // colour masks are two 64-bit words per vertex
constexpr int kMaxPlanes = 4;
constexpr int kMaxKinGroups = 8;
constexpr int kMaxEdgeColours = 64;  // colours of the distance constraints

// A contact against a frozen plane (q, n), as collision_constraint_t holds
// (src/physics/xpbd/collision_constraint.cpp:11-19): xyz of `q` is the contact
// point, q.w the vertex id (bit pattern); xyz of `n` the unit normal.
struct Contact {
    float4 q;
    float4 n;
};

// Device pointers of one scene.  Vertices are stored in the library's own
// (Morton) order; tets colour-major.
struct SceneDev {
    // vertices
    float4* xi;    // predicted / iterate position, w = inverse mass
    float4* xn;    // position at substep start (x == xn between substeps), w = inverse mass
    float4* v;     // velocity; w = 1 marks a kinematic vertex
    float4* acc;   // external acceleration (nullable)
    uint32_t n_verts;
    // kinematic vertices
    uint32_t* kin_vert;  // vertex id
    float4* kin_rel;     // x0 - centre (xyz), group id (w, as float)
    uint32_t n_kin;
    // tets, colour-major
    uint4* tet;
    float4* dm0;   // DmInv row 0, w = signed V0
    float4* dm1;   // DmInv row 1, w = mu
    float4* dm2;   // DmInv row 2, w = Lame lambda
    float* lam0;   // StVK multiplier / SNH deviatoric multiplier
    float* lam1;   // SNH hydrostatic multiplier
    uint8_t* model; // per slot: 0 StVK, 1 SNH (residual kernel)
    uint32_t n_tets;
    // surface and contacts
    uint32_t* surf;
    uint32_t n_surf;
    Contact* contacts;     // kMaxPlanes segments of n_surf, then body contacts
    float* contact_lam;
    uint32_t* counters;    // [0..kMaxPlanes) ground contacts per plane, [kMaxPlanes] body contacts
    uint32_t body_contact_cap;
    // distance constraints (distance_constraint.cpp:8-53), colour-major
    uint2* edge;           // vertex slots of the two ends
    float4* edge_p;        // x: rest length, y: compliance alpha, z: damping beta
    float* edge_lam;
    uint32_t n_edges;
    // control
    double* time;          // simulation time (s)
    int* err;              // first error code seen on the device
    unsigned* bar;         // grid barrier: [0] arrival count, [1] generation
    // wavefront mode: per-CTA count of finished colour phases, and the CTAs
    // whose tets share a vertex with each CTA's tets (CSR)
    uint32_t* prog;
    uint32_t* nb_start;
    uint32_t* nb;
    uint32_t* wave_start;  // [colour * (G + 1) + cta]: first entry of the CTA's tets in wave_idx
    uint32_t* wave_idx;    // tet slots, grouped by (colour, owning CTA)
    unsigned long long wait_ns;   // bound of every device wait (grid barrier, staging), then SBS_ETIMEOUT
    // reductions
    double* red_out;       // [4]: residual^2 (elastic), energy, residual^2 (contacts), spare
    float* partials;       // per-CTA partial sums for the residual kernel
};

struct KinGroup {
    float cx, cy, cz;
    float ax, ay, az;
    double omega;
};

struct Plane {
    float nx, ny, nz, d;
};

// Per-launch constants (kernel parameter space).
struct StepParams {
    float dt, inv_dt, inv_dt2;
    float stvk_alpha_tilde;      // alpha / dt^2
    float stvk_gamma;            // (alpha/dt^2)(beta dt^2)/dt
    int stvk_damping;            // 1 when beta != 0
    float contact_alpha_tilde;   // collision alpha / dt^2
    float gx, gy, gz;
    int gravity_mode;
    int n_colours;
    int first_tail;              // colours [first_tail, n_colours) run in one CTA
    int n_planes;                // environment slots: analytic planes, then SDF grids
    int n_analytic;              // slots [0, n_analytic) are planes
    int n_kin_groups;
    int substeps, iterations;
    int body_contacts;
    int has_acc;                 // 1 when an external acceleration field is set
    double dt_d;
    Plane planes[kMaxPlanes];
    SdfGrid grids[kMaxGrids];    // slot n_analytic + g
    KinGroup kin[kMaxKinGroups];
    uint32_t colour_start[kMaxColours + 1];
    uint32_t colour_split[kMaxColours];  // first SNH tet of each colour
    int n_edge_colours;
    uint32_t edge_start[kMaxEdgeColours + 1];
    int cl_flags;                // cluster mode, one warm-started substep: kClExternal | kClCarry | ...
    // kClJudge: the plain-solver judge inside the cluster kernel
    struct JudgeDev* judge;
    float4* judge_xpred;         // predicted positions (the plain start) of the substep
    uint32_t judge_chunk, judge_cap;
    int judge_substep;
};

// k_cluster_frame flags.  kClExternal: the substep's positions come
// predicted (and warm-started) in xi; the kernel runs that one substep's
// sweeps on them, takes the frame's contacts from the global contact list,
// and leaves prediction and velocity update to the global kernels.
// kClCarry: the elastic multipliers start from lam0/lam1, not from zero.
// kClContinue: the contact multipliers start from contact_lam (a further
// chunk of sweeps of the same substep), not from zero.
// kClJudge (with kClExternal | kClCarry, one cluster running the only group):
// the plain-solver judge runs inside the kernel - the warm start's residual
// against the plain start's (JudgeDev::r_plain0), the fallback, and sweeps
// in chunks of judge_chunk until the residual is at or below the target or
// the next chunk would pass judge_cap (iterations is then unused).
constexpr int kClExternal = 1;
constexpr int kClCarry = 2;
constexpr int kClContinue = 4;
constexpr int kClJudge = 8;
// kClCalibrate (one cluster running the only group, a plain frame): after
// each substep's sweeps the residual goes to JudgeDev::target[substep], and
// each substep's prediction to judge_xpred.
constexpr int kClCalibrate = 16;

// Device state of the plain-solver judge of warm-started substeps
// (warmstart.cu): residual targets from plain substeps, the running
// substep's residuals, and totals since the judge was set.
constexpr int kMaxJudgeSubsteps = 64;
struct JudgeDev {
    double target[kMaxJudgeSubsteps];  // plain residual after the full sweep count, per substep index
    double r_plain0;                   // residual of the plain start (predicted positions, zero multipliers)
    double r_start;                    // residual of the start the substep kept
    double r_now;                      // residual after the sweeps run so far
    uint32_t sweeps;                   // sweeps run in the current substep
    uint32_t fallback;                 // the current substep fell back to the plain start
    unsigned long long warm_substeps, calib_substeps, total_sweeps, fallbacks, capped;
    double sum_ratio, max_ratio;       // final residual / target over warm substeps
};

// What k_residual_final does with the residual it reduced (judge steps).
enum JudgeOpKind { kJudgeNone = 0, kJudgePlain0 = 1, kJudgeStart = 2, kJudgeChunk = 3, kJudgeCalib = 4 };
struct JudgeOp {
    int kind;
    int substep;                        // index into JudgeDev::target
    uint32_t chunk, cap;                // sweeps per check, most sweeps per substep
    JudgeDev* j;
    unsigned long long cond;            // cudaGraphConditionalHandle of the substep's sweep loop
};

// Kernel launchers (xpbd_kernels.cu).  All enqueue on `st`.
cudaError_t launch_detect_ground(const SceneDev& s, const StepParams& p, cudaStream_t st);
cudaError_t launch_predict(const SceneDev& s, const StepParams& p, int substep, cudaStream_t st);
cudaError_t launch_contacts(const SceneDev& s, const StepParams& p, int first_iter, cudaStream_t st);
cudaError_t launch_body_contacts(const SceneDev& s, const StepParams& p, int first_iter, cudaStream_t st);
cudaError_t launch_colour(const SceneDev& s, const StepParams& p, int colour, int first_iter, int block,
                          int grid, cudaStream_t st);
cudaError_t launch_tail(const SceneDev& s, const StepParams& p, int first_iter, int block, cudaStream_t st);
cudaError_t launch_finalize(const SceneDev& s, const StepParams& p, cudaStream_t st);
cudaError_t launch_edges(const SceneDev& s, const StepParams& p, int colour, int first_iter, cudaStream_t st);
cudaError_t launch_residual_ex(const SceneDev& s, const StepParams& p, int block, int grid, int cnt_base,
                               cudaStream_t st, int zero_lam = 0, const JudgeOp* op = nullptr);
cudaError_t launch_end_frame(const SceneDev& s, cudaStream_t st);
// stage: tet records copied into shared memory one colour phase ahead (bulk
// asynchronous copies per warp, csrc/xpbd_kernels.cu)
cudaError_t launch_persistent_frame(const SceneDev& s, const StepParams& p, int block, int grid,
                                    cudaStream_t st, int stage = 0);
cudaError_t persistent_occupancy(int block, int* ctas_per_sm, int stage = 0);
// State transfer (transfer_kernels.cu): o2n maps a global input vertex id to
// its library slot.
cudaError_t launch_gather_xyz(const float4* src, const uint32_t* o2n, uint32_t v0, uint32_t nv, float* out,
                              int check, int* bad, cudaStream_t st);
cudaError_t launch_check_finite(const float* in, uint64_t n, int* bad, cudaStream_t st);
cudaError_t launch_scatter_xyz(float4* dst, float4* dst2, const uint32_t* o2n, uint32_t v0, uint32_t nv,
                               const float* in, cudaStream_t st, const int* skip = nullptr);
// Wavefront variant of the frame kernel: every CTA owns the tets of one
// region of the mesh (s.wave_start / s.wave_idx) in every colour and, instead
// of a grid barrier per colour, waits until the CTAs it shares vertices with
// have finished the previous colour.  Needs s.prog zeroed before the launch.
cudaError_t wavefront_occupancy(int block, int* ctas_per_sm);
cudaError_t launch_wavefront_frame(const SceneDev& s, const StepParams& p, int block, int grid, cudaStream_t st);
cudaError_t launch_set_error(int* err, int code, cudaStream_t st);

}  // namespace sbs
