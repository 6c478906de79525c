/* sbs_gpu.h - C ABI of the GB300 XPBD solver (libsbs_gpu.so).
 *
 * The library replaces the per-frame hot path of Q-Minh/soft-body-simulator:
 * timestep_t::step (src/physics/timestep.cpp:20-70) together with the
 * gauss_seidel_solver_t it calls (src/physics/gauss_seidel_solver.cpp:8-37),
 * the constraint projections (src/physics/xpbd/green_constraint.cpp:49-158,
 * collision_constraint.cpp:21-48) and the contact generation of the
 * brute-force CD system (src/physics/collision/brute_force_cd_system.cpp:14-26,
 * bvh_model.cpp:30-100, xpbd/contact_handler.cpp:14-54).  Scene set-up, IO,
 * geometry and rendering stay on the host, unchanged.
 *
 * Conventions: plain C types only; every call returns an sbs_status;
 * positions are float (the reference's geometry_t stores float positions,
 * include/sbs/common/geometry.h) or double where the reference keeps double
 * state; arrays are tightly packed xyz triples.  One handle owns one CUDA
 * stream and all device memory of its scene; a handle must be used from one
 * host thread at a time.  sbs_gpu_step is asynchronous; every sbs_gpu_get_*
 * call synchronises the handle's stream.
 */
#ifndef SBS_GPU_H
#define SBS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum sbs_status {
    SBS_OK = 0,
    SBS_EINVAL = 1,    /* bad argument (null pointer, index out of range, bad size) */
    SBS_ECUDA = 2,     /* a CUDA runtime call failed */
    SBS_ETIMEOUT = 3,  /* a bounded device-side wait gave up (grid barrier) */
    SBS_ENAN = 4,      /* non-finite position detected */
    SBS_ESTATE = 5,    /* call not valid in the handle's current state */
    SBS_ENOMEM = 6,    /* device allocation failed */
    SBS_ECOLOUR = 7    /* constraint graph needs more colours than supported */
} sbs_status;

typedef enum sbs_model {
    SBS_MODEL_STVK = 0, /* Green-strain StVK energy constraint (green_constraint.cpp) */
    SBS_MODEL_SNH = 1   /* stable Neo-Hookean, two multipliers (Macklin & Mueller 2021) */
} sbs_model;

typedef enum sbs_gravity_mode {
    SBS_GRAVITY_ACCELERATION = 0, /* a = g on every free vertex */
    SBS_GRAVITY_FORCE = 1         /* f += g then a = f w, as timestep.cpp:39-40 */
} sbs_gravity_mode;

typedef enum sbs_exec_mode {
    SBS_EXEC_AUTO = 0,       /* pick with the built-in autotuner on the first step */
    SBS_EXEC_GRAPH = 1,      /* one kernel per phase, replayed as a CUDA graph */
    SBS_EXEC_PERSISTENT = 2, /* one cooperative kernel per frame, grid barriers */
    SBS_EXEC_CLUSTER = 3,    /* groups of bodies resident in the shared memory of a
                                thread-block cluster, cluster barriers between phases */
    SBS_EXEC_WAVEFRONT = 4   /* one cooperative kernel per frame; each CTA owns a slice
                                of every colour and waits only for the CTAs whose tets
                                share vertices with its own */
} sbs_exec_mode;

/* Solver parameters.  Defaults (sbs_gpu_params_default) follow
 * simulation_parameters_t (include/sbs/physics/xpbd/simulation_parameters.h:12-27). */
typedef struct sbs_gpu_params {
    double compliance;            /* alpha of the StVK energy constraint (1e-4) */
    double damping;               /* beta of the StVK energy constraint (0) */
    double collision_compliance;  /* alpha of contact constraints (1e-8) */
    double gravity[3];            /* (0, -9.81, 0) */
    int32_t gravity_mode;         /* sbs_gravity_mode */
    int32_t device;               /* CUDA device ordinal */
    int32_t exec_mode;            /* sbs_exec_mode */
    int32_t block_size;           /* threads per CTA of the projection kernels (0: auto) */
    int32_t ctas_per_sm;          /* persistent mode CTAs per SM (0: auto) */
    int32_t tail_threshold;       /* colours with <= this many tets run in one CTA (-1: the block
                                     size, then timed against 0 / 256 / 1024 / 4096 by the
                                     SBS_EXEC_AUTO autotuner) */
    int32_t body_contacts;        /* 0 off; 1 vertex-in-tet contacts between bodies (spatial
                                     hash); 2 also within a body (self contacts) */
    float hash_cell;              /* spatial hash cell size in metres (0: 2 x mean edge length) */
    uint32_t candidate_capacity;  /* >0: record up to this many broad-phase candidate pairs
                                     per detection for sbs_gpu_get_candidates */
    int32_t check_finite;         /* 1: sbs_gpu_get_* report SBS_ENAN on non-finite x */
    int32_t stage_records;        /* copy each colour's tet records into shared memory one phase
                                     ahead (bulk asynchronous copies) instead of loading them from
                                     global memory in the phase: 1 (default) in the cluster mode,
                                     2 also in the persistent mode (measured slower there: 24.5
                                     against 20.3 ms per frame of the 2.6M-tet block), 0 never */
    int32_t wait_limit_us;        /* bound of every device-side wait of the solver's kernels (grid
                                     barriers, staging waits) in microseconds, after which the
                                     kernel stops and the next synchronising call returns
                                     SBS_ETIMEOUT (0: 2 s) */
    int32_t colour_size_cap;      /* scenes that run in the global modes only: colours are
                                     rebalanced (more of them if needed) so that none holds more
                                     than this many tets - one tet per resident thread of the
                                     persistent kernel and phase.  0 (default): the device's
                                     resident threads (512 per SM); -1: no cap */
} sbs_gpu_params;

typedef struct sbs_gpu_material {
    int32_t model;     /* sbs_model */
    double young;      /* Young's modulus E (Pa) */
    double poisson;    /* Poisson ratio nu */
    double density;    /* kg/m^3, for lumped masses */
} sbs_gpu_material;

typedef struct sbs_gpu_stats {
    uint64_t frames;          /* frames stepped since finalize */
    uint64_t projections;     /* tet projections executed since finalize */
    uint32_t n_vertices, n_tets, n_colours, n_tail_colours;
    uint32_t n_contacts;      /* ground contacts of the last frame */
    uint32_t n_body_contacts; /* body-body contacts of the last frame */
    uint32_t body_contact_overflow; /* candidates dropped for lack of capacity */
    int32_t exec_mode;        /* mode in use after finalize */
    int32_t grid_ctas, block_size;
    double residual;          /* XPBD residual after the last substep (if evaluated) */
    double energy;            /* elastic energy after the last substep (if evaluated) */
    double last_frame_ms;     /* device time of the last timed frame (sbs_gpu_step_timed) */
    uint64_t kernel_launches; /* kernels run by sbs_gpu_step / step_timed since finalize
                                 (counted by the host as it enqueues them or their graph) */
    uint32_t cluster_phase_max_tets; /* cluster mode: most tets one CTA projects in one colour */
} sbs_gpu_stats;

typedef struct sbs_gpu sbs_gpu;

/* Fills *p with the defaults.  No reference counterpart (compile-time struct
 * simulation_parameters_t, simulation_parameters.h:10-28). */
sbs_status sbs_gpu_params_default(sbs_gpu_params* p);

/* Creates a handle (no scene yet).  Replaces constructing simulation_t and
 * timestep_t (include/sbs/physics/simulation.h:20-48, timestep.h:14-33). */
sbs_status sbs_gpu_create(const sbs_gpu_params* p, sbs_gpu** out);

/* Adds one tetrahedral body.  x0: rest positions [3*n_verts] (Dm, V0 and
 * lumped masses come from them); x_init: initial positions [3*n_verts] or
 * NULL for x0; tets: [4*n_tets] body-local vertex ids; mass: per-vertex mass
 * [n_verts] or NULL for lumped masses (density * |V0| / 4 per incident tet),
 * mass 0 pins a vertex.  Replaces tetrahedral_body_t's constructor
 * (src/physics/tetrahedral_body.cpp:30-83) plus the per-tet
 * green_constraint_t constructors in main.cpp:37-54 (green_constraint.cpp:11-47). */
sbs_status sbs_gpu_add_body(sbs_gpu* h, const double* x0, const double* x_init, uint32_t n_verts,
                            const uint32_t* tets, uint32_t n_tets, const sbs_gpu_material* mat,
                            const double* mass, int32_t* body_id);

/* A colouring of a body's tets (colours [n_tets of the body], each < 128)
 * for the sweep order, set before sbs_gpu_finalize: tets of one colour must
 * share no vertex (SBS_EINVAL at finalize otherwise).  When every tet of the
 * scene (or of a cluster group) has one and it needs no more colours than
 * the library's own colouring, it replaces that colouring; e.g. the lattice
 * colouring of a structured grid, which reaches the lower bound set by the
 * tets meeting at one vertex.  The reference has no counterpart: it projects
 * constraints in list order (gauss_seidel_solver.cpp:32-35). */
sbs_status sbs_gpu_set_tet_colours(sbs_gpu* h, int32_t body, const uint32_t* colours);
/* Pins vertices (w = 0), as setting particle_t::mass() = 0 does (main.cpp:158-165,
 * particle.cpp:39-49). */
sbs_status sbs_gpu_pin_vertices(sbs_gpu* h, int32_t body, const uint32_t* verts, uint32_t n);

/* Prescribed motion: verts follow x(t) = c + R(axis, omega t)(x0 - c) and have
 * w = 0.  No reference counterpart (the reference only pins). */
sbs_status sbs_gpu_add_kinematic_rotation(sbs_gpu* h, int32_t body, const uint32_t* verts,
                                          uint32_t n, const double center[3],
                                          const double axis[3], double omega);

/* Per-vertex external acceleration field [3*n_verts] (m/s^2), added in the
 * prediction.  No reference counterpart (particle_t::f is zeroed every substep,
 * timestep.cpp:55). */
sbs_status sbs_gpu_set_external_acceleration(sbs_gpu* h, int32_t body, const float* acc);

/* Adds the analytic plane SDF n.x + d = 0 (normal is normalised).  Replaces
 * sdf_model_t::from_plane (src/physics/collision/sdf_model.cpp:52-64) used with
 * environment_body_t in main.cpp:60-72. */
sbs_status sbs_gpu_add_ground_plane(sbs_gpu* h, const double n[3], double d);

/* Initial velocity of every vertex of a body (physics_body_info::velocity of
 * a scene object, load_scene.cpp:246-250).  Before finalize. */
sbs_status sbs_gpu_set_body_velocity(sbs_gpu* h, int32_t body, const double v[3]);

/* read_ply (src/io/ply.cpp): vertex x y z (kept as float, as geometry_t does),
 * `face` elements with 3 indices -> triangles, `tet` elements with 4 -> tets;
 * ascii, binary_little_endian or binary_big_endian.  Any output may be NULL
 * (counts only); capacities are in vertices / triangles / tets.  Host only. */
sbs_status sbs_io_read_ply(const char* path, float* positions, uint32_t cap_verts, uint32_t* n_verts,
                           uint32_t* tris, uint32_t cap_tris, uint32_t* n_tris, uint32_t* tets, uint32_t cap_tets,
                           uint32_t* n_tets);
/* load_scene (src/io/load_scene.cpp:83-365) into a handle before finalize:
 * every "environment" entry that is a collideable PLY triangle mesh becomes
 * an environment SDF (sbs_gpu_add_environment_mesh over the mesh's bounds
 * grown by env_margin metres on every side - the depth below a floor in which
 * contacts are found - with env_cells cells per axis); every "objects" entry
 * with a PLY tet mesh becomes
 * a body with `material` (its density replaced by "physics"."mass", the
 * reference's mass density) and initial velocity "physics"."velocity".  Both
 * are first rescaled into their "box" and moved by their "translation" as the
 * reference does.  Paths are relative to the JSON file.  Lights, colours and
 * non-PLY assets are skipped.  *first_body / *n_bodies: the bodies added. */
sbs_status sbs_gpu_load_scene(sbs_gpu* h, const char* json_path, const sbs_gpu_material* material,
                              const uint32_t env_cells[3], double env_margin, int32_t* first_body,
                              int32_t* n_bodies);

/* Signed-distance grid of an environment body: node values [nx * ny * nz],
 * index (k * ny + j) * nx + i at origin + (i, j, k) * spacing, evaluated by
 * trilinear interpolation with the interpolant's gradient.  Surface vertices
 * with sd < 0 get the contact of bvh_model.cpp:72-94 (n = normalised
 * gradient, q = p + |sd| n); outside the grid there is no contact.  Up to 2
 * grids (of either kind); planes and grids together at most 4, planes first.
 * Before finalize; not with SBS_EXEC_CLUSTER. */
sbs_status sbs_gpu_add_sdf_grid(sbs_gpu* h, const float* values, const uint32_t nodes[3], const double origin[3],
                                const double spacing[3]);
/* The cubic Lagrange grid sdf_model_t interpolates
 * (src/physics/collision/sdf_model.cpp:66-75, a Discregrid
 * CubicLagrangeDiscreteGrid built at environment_body.cpp:72-73): cells[3]
 * cells of size `spacing` from `origin`, each the 32-node serendipity
 * element (Koschier et al. 2017; corners and the points at 1/3 and 2/3 of
 * every edge), the interpolant's gradient as normal.  values: the (cells+1)
 * vertices per axis, index (k * ny + j) * nx + i; then 2 values per x-edge
 * (edge (i, j, k), i < cells[0], index (k * ny + j) * cells[0] + i, the node
 * at 1/3 first), per y-edge ((k * cells[1] + j) * nx + i) and per z-edge
 * ((k * ny + j) * nx + i, k < cells[2]), with nx, ny the vertices per axis.
 * Otherwise as sbs_gpu_add_sdf_grid. */
sbs_status sbs_gpu_add_sdf_grid_cubic(sbs_gpu* h, const float* values, const uint32_t cells[3], const double origin[3],
                                      const double spacing[3]);
/* environment_body_t's constructor (src/physics/environment_body.cpp:12-78) for
 * a triangle mesh (outward winding): the domain grown over the mesh vertices
 * and padded as that constructor does, `cells` cells per axis, node values from
 * sbs_gpu_sdf_cubic_from_mesh, added with sbs_gpu_add_sdf_grid_cubic. */
sbs_status sbs_gpu_add_environment_mesh(sbs_gpu* h, const double* verts, uint32_t n_verts, const uint32_t* tris,
                                        uint32_t n_tris, const double domain_lo[3], const double domain_hi[3],
                                        const uint32_t cells[3]);
/* Host only (no handle, no GPU): signed distance of a triangle mesh at the
 * (cells + 1)^3 nodes of the box [lo, hi], into values (layout as above).
 * Closest point per triangle (Ericson 2005, 5.1.5), sign from the angle-weighted
 * pseudonormal (Baerentzen & Aanaes 2005); brute force over triangles. */
sbs_status sbs_gpu_sdf_from_mesh(const double* verts, uint32_t n_verts, const uint32_t* tris, uint32_t n_tris,
                                 const double lo[3], const double hi[3], const uint32_t cells[3], float* values);
/* Host only: the values of the cubic grid of sbs_gpu_add_sdf_grid_cubic
 * (layout there) for a triangle mesh over the box [lo, hi]. */
sbs_status sbs_gpu_sdf_cubic_from_mesh(const double* verts, uint32_t n_verts, const uint32_t* tris, uint32_t n_tris,
                                       const double lo[3], const double hi[3], const uint32_t cells[3],
                                       float* values);

/* Distance constraints: n rows of ids [4n] = (b1, b2, v1, v2) - body and
 * body-local vertex of each end, the order of distance_constraint_t's
 * constructor (src/physics/xpbd/distance_constraint.cpp:8-22) - with
 * compliance alpha and damping beta; rest length |x0_1 - x0_2|.  Projected by
 * distance_constraint_t::project_positions (:24-53) in every iteration after
 * the tet constraints, in their own colours (sbs_gpu_get_distance_order).
 * Coincident ends, where the reference divides by zero, leave a constraint
 * unchanged.  Before finalize; not with SBS_EXEC_CLUSTER (the other modes run
 * them). */
sbs_status sbs_gpu_add_distance_constraints(sbs_gpu* h, const uint32_t* ids, uint32_t n, double alpha,
                                            double beta);

/* Colours the constraint graph, orders tets by (colour, Morton code), uploads
 * the scene and selects the execution mode.  After this the scene is fixed.
 * No single reference counterpart: it replaces building the constraint list
 * and the brute-force CD system (main.cpp:37-54, :74-88). */
sbs_status sbs_gpu_finalize(sbs_gpu* h);

/* One frame: contacts from the frame-start positions, then `substeps` times
 * predict -> `iterations` Gauss-Seidel sweeps -> velocity update.  Replaces
 * timestep_t::step (timestep.cpp:20-70) with gauss_seidel_solver_t::solve
 * (gauss_seidel_solver.cpp:8-37) installed as the solver.  Asynchronous. */
sbs_status sbs_gpu_step(sbs_gpu* h, double frame_dt, uint32_t substeps, uint32_t iterations);

/* As sbs_gpu_step, bracketed by CUDA events; waits and stores the frame's
 * device time in stats.last_frame_ms. */
sbs_status sbs_gpu_step_timed(sbs_gpu* h, double frame_dt, uint32_t substeps, uint32_t iterations);
/* Test hook for the timeout path, no reference counterpart: the next frame
 * of the persistent mode starts its grid-barrier arrival count one arrival
 * short, so its first grid barrier never completes; every CTA gives up after
 * wait_limit_us, the kernel returns, and the next synchronising call
 * reports SBS_ETIMEOUT.  That frame is left incomplete; the error is cleared
 * when reported and later frames run normally.  SBS_ESTATE unless the
 * handle runs the persistent mode. */
sbs_status sbs_gpu_withhold_barrier_arrival(sbs_gpu* h);

/* The solver seam alone: resets every multiplier and runs `iterations`
 * sweeps (contacts first, then the elastic colours) on the current predicted
 * positions.  Replaces solver_t::solve (include/sbs/physics/solver.h:16). */
sbs_status sbs_gpu_solve(sbs_gpu* h, double dt, uint32_t iterations);

/* The prediction and velocity-update halves of a substep (timestep.cpp:35-43,
 * :48-57), and contact detection alone (cd_system_t::execute, cd_system.h:32). */
sbs_status sbs_gpu_predict(sbs_gpu* h, double dt);
sbs_status sbs_gpu_update_velocities(sbs_gpu* h, double dt);
sbs_status sbs_gpu_detect_contacts(sbs_gpu* h);

/* Evaluates the XPBD residual sqrt(sum (C + alpha~ lambda)^2) over elastic
 * and active contact constraints, and the elastic energy, at the current
 * predicted positions with compensated (Kahan) FP32 sums.  Writes both. */
sbs_status sbs_gpu_residual(sbs_gpu* h, double dt, double* residual, double* energy);

/* State transfer for one body, or with body = -1 for the whole scene in
 * global vertex order (bodies in add order), as simulation_t::particles()
 * holds it (host buffers; pinned memory is fastest).
 * x: positions [3*n_verts], v: velocities [3*n_verts]; either may be NULL.
 * set_state writes x into x, xn and xi, as a particle_t's state after a frame.
 * The gpu_timestep_t adapter calls these around sbs_gpu_step. */
sbs_status sbs_gpu_set_state(sbs_gpu* h, int32_t body, const float* x, const float* v);
sbs_status sbs_gpu_get_state(sbs_gpu* h, int32_t body, float* x, float* v);
/* Predicted/iterate positions xi of one body (-1: whole scene) [3*n_verts]. */
sbs_status sbs_gpu_get_predicted(sbs_gpu* h, int32_t body, float* xi);
sbs_status sbs_gpu_set_predicted(sbs_gpu* h, int32_t body, const float* xi);

/* Introspection for parity checks.
 * get_tet_order: order[k] = global tet id (bodies concatenated in add order)
 *   projected k-th in a sweep; offsets: n_colours + 1 entries.
 * get_lambdas: [2*n_tets] in global tet order (StVK/deviatoric, hydrostatic).
 * get_contacts: vertex ids [cap] and (q, n) [6*cap] of the current frame's
 *   ground contacts, sorted by (plane, vertex); returns the count in *n. */
sbs_status sbs_gpu_get_tet_order(sbs_gpu* h, uint32_t* order, uint32_t* offsets, uint32_t cap_offsets,
                                 uint32_t* n_colours);
sbs_status sbs_gpu_get_lambdas(sbs_gpu* h, float* lambdas);
/* Projection order of the distance constraints (input indices, colour-major)
 * and colour offsets [n_colours + 1]; their multipliers in input order. */
sbs_status sbs_gpu_get_distance_order(sbs_gpu* h, uint32_t* order, uint32_t* offsets, uint32_t cap_offsets,
                                      uint32_t* n_colours);
sbs_status sbs_gpu_get_distance_lambdas(sbs_gpu* h, float* lambdas);
sbs_status sbs_gpu_get_contacts(sbs_gpu* h, uint32_t* verts, float* qn, uint32_t cap, uint32_t* n);
sbs_status sbs_gpu_get_masses(sbs_gpu* h, float* inv_mass);
/* Broad-phase candidate pairs of the last contact detection (needs
 * params.candidate_capacity > 0), as (global vertex id << 32 | global tet id),
 * sorted ascending; *n receives the total count (may exceed cap).  No
 * reference counterpart: the reference's CD has no body-body pairs
 * (contact_handler.cpp:17 handles SDF contacts only). */
sbs_status sbs_gpu_get_candidates(sbs_gpu* h, uint64_t* pairs, uint64_t cap, uint64_t* n);
sbs_status sbs_gpu_get_surface(sbs_gpu* h, uint32_t* verts, uint32_t cap, uint32_t* n);

/* Visual model of a body: the boundary triangle mesh tetrahedral_mesh_boundary_t
 * builds (src/physics/tetrahedral_mesh_boundary.cpp:76-120) - faces with != 2
 * incident tets, in the order and winding of their first appearance over the
 * tets (input order) and their faces_copy faces (src/physics/topology.cpp:335-342);
 * surface vertices numbered by first appearance.  triangles [3 * n_triangles]
 * holds surface-vertex ids, vertex_map [n_vertices] the body-local vertex of
 * each surface vertex (tetrahedral_mesh_boundary_t::from_surface_vertex).
 * Either array may be NULL (counts only). */
sbs_status sbs_gpu_get_surface_mesh(sbs_gpu* h, int32_t body, uint32_t* triangles, uint32_t cap_triangles,
                                    uint32_t* n_triangles, uint32_t* vertex_map, uint32_t cap_vertices,
                                    uint32_t* n_vertices);
/* tetrahedral_body_t::update_visual_model (src/physics/tetrahedral_body.cpp:157-165)
 * on the device: each surface vertex takes its vertex's position, and the
 * vertex normals get compute_normals' update (tetrahedral_mesh_boundary.cpp:122-145):
 * add (p2 - p1) x (p3 - p1) of every incident boundary triangle, in triangle
 * order, then normalise.  The reference never clears the normals, so each
 * update adds to the previous normal: accumulate_normals = 1 keeps that
 * behaviour (the state starts at zero and finalize runs the constructor's
 * first update), 0 starts from zero.  When vertex_buffer is not NULL, surface
 * vertex i's position and normal are written to vertex_buffer[i * stride + 0..5]
 * (stride >= 6 floats; 9 is the reference's render layout position, normal,
 * colour, whose colour floats are left untouched).  vertex_buffer may be device
 * memory of the handle's device (written by the kernel, no host copy) or host
 * memory.  Returns when the buffer is written. */
sbs_status sbs_gpu_update_surface(sbs_gpu* h, int32_t body, int32_t accumulate_normals, float* vertex_buffer,
                                  uint32_t stride);
sbs_status sbs_gpu_get_stats(sbs_gpu* h, sbs_gpu_stats* st);

/* Host-only (no GPU needed): the Gauss-Seidel sweep order the solver uses
 * for this tet list - tets coloured so that no two tets of a colour share a
 * vertex, colours by decreasing size, tets of a colour by model then by the
 * Morton code of the rest centroid.  x0 [3*n_verts], tets [4*n_tets],
 * models [n_tets] or NULL (all StVK); colours [n_tets] or NULL: a caller's
 * colouring as sbs_gpu_set_tet_colours takes it (-1: none); order [n_tets];
 * offsets [n_colours+1]
 * (cap_offsets entries available).  For several bodies pass them
 * concatenated in add order.  The reference has no counterpart: it projects
 * constraints in list order (gauss_seidel_solver.cpp:32-35); permuting its
 * list to this order gives the same sweep as the GPU. */
sbs_status sbs_gpu_plan_sweep(const double* x0, uint32_t n_verts, const uint32_t* tets, uint32_t n_tets,
                              const int32_t* models, const int32_t* colours, uint32_t* order, uint32_t* offsets,
                              uint32_t cap_offsets, uint32_t* n_colours);

/* Plane-contact detection for callers that cannot allocate device memory.
 * No counterpart in the reference (which has no GPU code); it is the ground
 * contact rule of the solver (surface vertex with n.x + d < 0 becomes a
 * contact at q = x + |n.x + d| n) offered as one call on buffers the caller
 * already owns, for hosts that hand out every device byte through their own
 * allocator or budget, code running inside CUDA stream capture, and real-time
 * loops that cannot take an allocation's implicit synchronisation.
 * All pointers are DEVICE pointers: x [3*n_verts] float positions,
 * surface [n_surface] vertex ids, contact_verts [n_surface] and
 * contact_points [3*n_surface] outputs (contacts in the order of `surface`),
 * count [1] output.  n_surface <= 1,048,576 (SBS_EINVAL beyond).  Surface
 * ids >= n_verts are skipped (never read, never reported), so with such ids
 * the count can be lower than the solver's.  Enqueued on `stream` (a
 * cudaStream_t; NULL for the default stream), asynchronous.  A CUDA error
 * already pending on the calling thread is returned as SBS_ECUDA before
 * anything is enqueued.  Working memory is a 32 KB static device array
 * shared by every call on a device: calls that overlap on the GPU race; the
 * first call on a device looks the array up (cudaGetSymbolAddress) and keeps
 * the address, so make that first call outside any stream capture, and do
 * not use this call after a cudaDeviceReset in the same process.  Allocates
 * nothing. */
sbs_status sbs_gpu_plane_contacts_noalloc(const float* x, uint32_t n_verts, const uint32_t* surface,
                                          uint32_t n_surface, const double normal[3], double d,
                                          uint32_t* contact_verts, float* contact_points, uint32_t* count,
                                          void* stream);

/* ---- Learned warm start: per-vertex MLP 16 -> 128 -> 128 -> 128 -> 3 (SiLU),
 * BF16 tensor-core GEMMs with FP32 accumulate, FP32 master weights, Adam.
 * No reference counterpart (the reference always starts its sweeps from the
 * predicted positions, timestep.cpp:35-45).  Parameters are laid out
 * W1[128][16] b1 W2[128][128] b2 W3[128][128] b3 W4[3][128] b4 (35,587 floats).
 * Features per vertex (16): inertial displacement xi - x (3), mean deformation
 * gradient of incident tets, row-major (9), external acceleration (3), pin flag
 * (1); output: displacement correction (3).  Inputs are normalised as
 * (x - mean) / std and outputs multiplied by out_scale inside the network. */
typedef struct sbs_mlp sbs_mlp;
uint32_t sbs_mlp_param_count(void);
sbs_status sbs_mlp_create(int32_t device, uint64_t seed, sbs_mlp** out);
sbs_status sbs_mlp_destroy(sbs_mlp* m);
const char* sbs_mlp_last_error(const sbs_mlp* m);
sbs_status sbs_mlp_get_params(sbs_mlp* m, float* params);
sbs_status sbs_mlp_set_params(sbs_mlp* m, const float* params);
sbs_status sbs_mlp_set_normalization(sbs_mlp* m, const float* in_mean, const float* in_std, const float* out_scale);
/* Host buffers: x [n*16] raw features -> y [n*3] raw outputs. */
sbs_status sbs_mlp_forward(sbs_mlp* m, const float* x, uint32_t n, float* y);
/* As sbs_mlp_forward with the implementation chosen: 0 the fused tcgen05
 * kernel (the default; weights resident in shared memory, accumulators in
 * tensor memory), 1 the per-layer GEMMs that training uses (engine chosen by
 * sbs_mlp_set_gemm). */
sbs_status sbs_mlp_forward_path(sbs_mlp* m, const float* x, uint32_t n, float* y, int32_t path);
/* The same on device buffers of the network's device (x [n*16], y [n*3]);
 * with ms != NULL the kernels' device time in milliseconds (CUDA events on
 * the network's stream).  Returns when y is written. */
sbs_status sbs_mlp_forward_device(sbs_mlp* m, const float* x, uint32_t n, float* y, int32_t path, float* ms);
/* Host buffers: loss = mean over rows of ||(y - t) / out_scale||^2 and its
 * gradient w.r.t. all parameters (for gradient checks). */
sbs_status sbs_mlp_loss_grad(sbs_mlp* m, const float* x, const float* t, uint32_t n, float* loss, float* grad);
/* Training set upload (host buffers x [n*16], t [n*3]) and `steps` Adam steps
 * on random batches of `batch` rows; *loss = loss of the last batch. */
sbs_status sbs_mlp_set_dataset(sbs_mlp* m, const float* x, const float* t, uint32_t n);
sbs_status sbs_mlp_train(sbs_mlp* m, uint32_t steps, uint32_t batch, float lr, uint64_t seed, float* loss);
/* Engine of the per-layer GEMMs (training, loss_grad, forward path 1): 0 the
 * tcgen05 kernels (default; TMEM accumulators, split-K weight gradients summed
 * in a fixed order), 1 the warp-level mma.sync kernels.  Each engine gives the
 * same result bit for bit on every run; the two differ in summation order.
 * loss_grad and train return SBS_ETIMEOUT when a tensor-core wait expired. */
sbs_status sbs_mlp_set_gemm(sbs_mlp* m, int32_t engine);

/* Attaches (m != NULL) or detaches the warm-start network.  While attached,
 * every substep of sbs_gpu_step runs predict -> features -> MLP ->
 * `fit_sweeps` (1..16) fit sweeps that turn the guessed displacement (the
 * previous substep's solve displacement plus the network's correction) into
 * multipliers (colour order, each constraint's increment best matching the
 * displacement still missing at its vertices) -> `iterations` sweeps
 * continuing from those multipliers.  fit_sweeps = 0 is the carry start: the
 * free vertices move by the guessed displacement and the elastic multipliers
 * keep the values the previous substep's solve ended with (zero when there is
 * no previous substep).  The previous substep's displacement is known when
 * its features were computed and the state was not replaced since
 * (set_state / set_predicted / a frame without the network reset it to 0).
 * Do not train the same network while it is attached. */
sbs_status sbs_gpu_set_warm_start(sbs_gpu* h, sbs_mlp* m, uint32_t fit_sweeps);
/* The plain solver as the judge of warm-started substeps (the reference
 * always runs the plain sweep count from the predicted positions with zero
 * multipliers, gauss_seidel_solver.cpp:8-37; its residual is the yardstick).
 * With check_every > 0 and a network attached, every substep of
 * sbs_gpu_step runs on the device:
 *   1. the residual of the plain start (predicted positions, zero
 *      multipliers) and of the warm start; a warm start whose residual is
 *      not below the plain start's is discarded and the substep continues
 *      from the plain start (a fallback);
 *   2. sweeps in chunks of check_every, each followed by the residual, until
 *      the residual is at or below the target or the next chunk would pass
 *      max_sweeps (0: the step's `iterations`).
 * The target of substep k of a frame is the residual that a plain substep k
 * (the step's `iterations` sweeps) reached in the last calibration frame: the
 * first judged frame and then every calibrate_every-th frame (0: the first
 * only) run plain and record their residuals.  fixed_target > 0 sets the
 * target of every substep instead, and then no frame calibrates.  Residual
 * as sbs_gpu_residual (compensated FP32 sums of (C + alpha~ lambda)^2 over
 * the elastic, distance and contact constraints).  The loop is a conditional
 * node of the frame's CUDA graph whose condition the device sets, so a frame
 * still needs no host round trip.  check_every = 0 turns the judge off.
 * Calling this resets the totals of sbs_gpu_get_warm_stats. */
sbs_status sbs_gpu_set_warm_judge(sbs_gpu* h, uint32_t check_every, uint32_t max_sweeps, uint32_t calibrate_every,
                                  double fixed_target);
typedef struct sbs_gpu_warm_stats {
    uint64_t warm_substeps;         /* judged warm-started substeps run */
    uint64_t calibration_substeps;  /* plain substeps run to record targets */
    uint64_t sweeps;                /* sweeps of the judged substeps, in total */
    uint64_t fallbacks;             /* warm starts discarded for the plain start */
    uint64_t capped;                /* substeps that stopped at max_sweeps above their target */
    double mean_residual_ratio;     /* final residual / target, mean over judged substeps */
    double max_residual_ratio;      /* and its maximum */
    double last_target;             /* target of substep 0 */
    double last_residual;           /* final residual of the last judged substep */
} sbs_gpu_warm_stats;
/* Totals of the judge since sbs_gpu_set_warm_judge (synchronises). */
sbs_status sbs_gpu_get_warm_stats(sbs_gpu* h, sbs_gpu_warm_stats* out);
/* The warm-start half of a substep on its own, after sbs_gpu_predict. */
sbs_status sbs_gpu_warm_start_init(sbs_gpu* h, double dt);
/* As sbs_gpu_solve; with reset_lambda = 0 the sweeps continue from the
 * current multipliers (after sbs_gpu_warm_start_init) instead of resetting
 * them as constraint_t::prepare_for_projection does (constraint.cpp:12-16). */
sbs_status sbs_gpu_solve_ex(sbs_gpu* h, double dt, uint32_t iterations, int32_t reset_lambda);
/* Features of every vertex at the current predicted state, host [16 * n_vertices]
 * in global vertex order (training data).  Call it once per substep, after
 * sbs_gpu_predict: it also records the prediction that the next substep's
 * previous-displacement features are measured from. */
sbs_status sbs_gpu_get_features(sbs_gpu* h, float* feat);

/* Frees every device resource of the handle. */
sbs_status sbs_gpu_destroy(sbs_gpu* h);

/* Human-readable text of a status code (static storage). */
const char* sbs_gpu_status_string(sbs_status s);

/* Text of the last error recorded on the handle (static per handle). */
const char* sbs_gpu_last_error(const sbs_gpu* h);

#ifdef __cplusplus
}
#endif

#endif /* SBS_GPU_H */
