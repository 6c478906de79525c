// XPBD substep kernels for sm_103a.
//
// One frame = contact detection, then per substep: predict -> iterations x
// (contact phase, elastic colour phases) -> velocity update.  This is the loop
// of timestep_t::step (src/physics/timestep.cpp:20-70) with
// gauss_seidel_solver_t::solve (src/physics/gauss_seidel_solver.cpp:8-37).
// Gauss-Seidel order is kept exactly: tets of one colour share no vertex, so
// running a colour in parallel equals running it in any sequential order, and
// colours run one after the other.  No atomics touch positions or multipliers.
//
// Two drivers share the phase code:
//  * per-phase kernels, recorded once into a CUDA graph per frame shape;
//  * one cooperative persistent kernel per frame, phases separated by a grid
//    barrier whose wait is bounded in time (SBS_ETIMEOUT on expiry).
#include <cuda_runtime.h>
#include <stdint.h>

#include "xpbd_internal.cuh"
#include "launch_count.cuh"
#include "xpbd_math.cuh"

namespace sbs {

uint64_t& launch_counter() {
    static thread_local uint64_t n = 0;
    return n;
}

constexpr int kErrTimeout = 3;  // SBS_ETIMEOUT

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_relaxed(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Grid-wide barrier for a cooperative launch.  bar[0] counts arrivals over
// the whole launch (zeroed by the host before it); barrier number k of the
// launch completes when the count reaches k * gridDim.x, so thread 0 of each
// CTA adds one with release semantics and waits, with acquire loads, for the
// count to reach its target - one round trip, no reset.  No extra fences:
// the CTA barrier before the release add and after the acquire load carries
// the other threads' writes and reads (release and acquire are cumulative in
// the PTX memory model); dropping the two __threadfence calls took 18% off a
// frame of the 98k-tet beam in this mode.  A wait longer than `limit_ns`
// (SceneDev::wait_ns) records SBS_ETIMEOUT.  Returns false when the kernel must stop (timeout
// here or an error recorded by another CTA).
__device__ __forceinline__ void grid_arrive(unsigned* bar, unsigned& target) {
    target += gridDim.x;
    __syncthreads();
    if (threadIdx.x == 0) red_release_add(bar, 1u);
}

__device__ __forceinline__ bool grid_wait(unsigned* bar, int* err, unsigned target,
                                          unsigned long long limit_ns) {
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned long long t0 = global_ns();
        unsigned spins = 0;
        while (ld_acquire(bar) < target) {
            if ((++spins & 63u) == 0) {
                if (ld_relaxed(err) != 0) { ok = 0; break; }
                if (global_ns() - t0 > limit_ns) {
                    atomicCAS(err, 0, kErrTimeout);
                    ok = 0;
                    break;
                }
            }
        }
        if (ok && ld_relaxed(err) != 0) ok = 0;
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// grid_arrive + grid_wait.  Loads of read-only data issued between the two
// overlap the wait without holding back the CTA's arrival.
__device__ __forceinline__ bool grid_barrier(unsigned* bar, int* err, unsigned& target,
                                             unsigned long long limit_ns) {
    grid_arrive(bar, target);
    return grid_wait(bar, err, target, limit_ns);
}

// Work mapping for one phase: 32-item chunks dealt round-robin over CTAs
// first, so a small colour spreads over many SMs; lanes of a warp take
// consecutive items (coalesced SoA loads).
template <typename Fn>
__device__ __forceinline__ void for_each_spread(uint32_t begin, uint32_t end, Fn&& fn) {
    const uint32_t lane = threadIdx.x & 31u, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    const uint32_t n = end - begin;
    const uint32_t chunks = (n + 31u) >> 5;
    for (uint32_t c = wib * gridDim.x + blockIdx.x; c < chunks; c += gridDim.x * wpb) {
        const uint32_t i = (c << 5) + lane;
        if (i < n) fn(begin + i);
    }
}

template <typename Fn>
__device__ __forceinline__ void for_each_vertex(uint32_t n, Fn&& fn) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) fn(i);
}

// ---------------------------------------------------------------------------
// Phases

// Prediction (timestep.cpp:35-43) for vertex i, fused with the prescribed
// motion of kinematic vertices (v.w = 1 + group; rest offset in acc[i]).
__device__ __forceinline__ void predict_vertex(const SceneDev& s, const StepParams& p, uint32_t i,
                                               double t_next, int has_acc) {
    float4 v = s.v[i];
    const float4 x = s.xn[i];
    if (v.w != 0.0f) {
        const int g = (int)v.w - 1;
        const KinGroup k = p.kin[g];
        const float4 rel = s.acc[i];
        float sn, cs;
        sincosf((float)(k.omega * t_next), &sn, &cs);
        const f3 a = mk(k.ax, k.ay, k.az), r = mk(rel.x, rel.y, rel.z);
        const f3 rr = r * cs + cross(a, r) * sn + a * (dot(a, r) * (1.0f - cs));
        s.xi[i] = make_float4(k.cx + rr.x, k.cy + rr.y, k.cz + rr.z, x.w);
        return;
    }
    const float w = x.w;
    float ax = 0.f, ay = 0.f, az = 0.f;
    if (w > 0.0f) {
        if (p.gravity_mode == 1) { ax = p.gx * w; ay = p.gy * w; az = p.gz * w; }
        else { ax = p.gx; ay = p.gy; az = p.gz; }
        if (has_acc) {
            const float4 e = s.acc[i];
            ax += e.x; ay += e.y; az += e.z;
        }
    }
    v.x += ax * p.dt;
    v.y += ay * p.dt;
    v.z += az * p.dt;
    s.v[i] = v;
    s.xi[i] = make_float4(x.x + v.x * p.dt, x.y + v.y * p.dt, x.z + v.z * p.dt, w);
}

// Velocity update (timestep.cpp:48-57): x = xi; v = (x - xn)/dt; xn = x.
__device__ __forceinline__ void finalize_vertex(const SceneDev& s, const StepParams& p, uint32_t i) {
    const float4 a = s.xi[i];
    const float4 b = s.xn[i];
    float4 v = s.v[i];
    v.x = (a.x - b.x) * p.inv_dt;
    v.y = (a.y - b.y) * p.inv_dt;
    v.z = (a.z - b.z) * p.inv_dt;
    s.v[i] = v;
    s.xn[i] = a;
}

// Environment contact detection for item k of (environment slots x surface
// vertices): bvh_model.cpp:72-94 - a surface vertex with signed distance
// sd < 0 gets the contact n = normalised gradient, q = p + |sd| n - with the
// plane SDF of sdf_model.cpp:52-64 or a signed-distance grid.
__device__ __forceinline__ void detect_item(const SceneDev& s, const StepParams& p, uint32_t k) {
    const uint32_t plane = k / s.n_surf;
    const uint32_t vi = s.surf[k - plane * s.n_surf];
    const float4 x = s.xn[vi];
    float sd = 0.0f, nx = 0.0f, ny = 0.0f, nz = 0.0f;
    bool hit;
    if ((int)plane < p.n_analytic) {
        const Plane pl = p.planes[plane];
        sd = pl.nx * x.x + pl.ny * x.y + pl.nz * x.z + pl.d;
        nx = pl.nx; ny = pl.ny; nz = pl.nz;
        hit = sd < 0.0f;
    } else {
        float gx, gy, gz;
        hit = sdf_eval(p.grids[plane - p.n_analytic], x.x, x.y, x.z, sd, gx, gy, gz) && sd < 0.0f;
        if (hit) {
            const float l = sqrtf(gx * gx + gy * gy + gz * gz);
            hit = l > 0.0f;
            if (hit) { nx = gx / l; ny = gy / l; nz = gz / l; }
        }
    }
    // one atomic per (warp, slot): a warp may straddle two slots
    const unsigned act = __activemask();
    const unsigned same = __match_any_sync(act, plane);
    const unsigned mask = __ballot_sync(act, hit) & same;
    if (!hit) return;
    const unsigned lane = threadIdx.x & 31u;
    const int leader = __ffs(mask) - 1;
    unsigned base = 0;
    if ((int)lane == leader) base = atomicAdd(&s.counters[plane], (unsigned)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    const unsigned rank = __popc(mask & ((1u << lane) - 1u));
    if (base + rank >= s.n_surf) return;  // cannot happen with reset counters; never write past the segment
    const float ad = fabsf(sd);
    Contact c;
    c.q = make_float4(x.x + nx * ad, x.y + ny * ad, x.z + nz * ad, __uint_as_float(vi));
    c.n = make_float4(nx, ny, nz, 0.0f);
    s.contacts[(size_t)plane * s.n_surf + base + rank] = c;
}

// collision_constraint_t::project_positions (collision_constraint.cpp:21-41).
__device__ __forceinline__ void project_contact(const SceneDev& s, const StepParams& p, uint32_t ci,
                                                bool first) {
    const Contact c = s.contacts[ci];
    const uint32_t vi = __float_as_uint(c.q.w);
    float lam = first ? 0.0f : s.contact_lam[ci];
    float4 x = __ldcg(&s.xi[vi]);
    const float C = (x.x - c.q.x) * c.n.x + (x.y - c.q.y) * c.n.y + (x.z - c.q.z) * c.n.z;
    if (C < 0.0f) {
        const float w = x.w;
        const float dl = -(C + p.contact_alpha_tilde * lam) / (w + p.contact_alpha_tilde);
        lam += dl;
        x.x += w * c.n.x * dl;
        x.y += w * c.n.y * dl;
        x.z += w * c.n.z * dl;
        s.xi[vi] = x;
    }
    s.contact_lam[ci] = lam;
}

// The part of a tet's record that no other tet's projection changes: indices,
// rest data and its own multipliers (written only by this tet's projection,
// in an earlier sweep).  None of it depends on positions, so the persistent
// kernel loads a thread's next tet while it waits at the grid barrier that
// precedes the projection.
struct TetRec {
    uint4 id;
    float4 a, b, c;   // DmInv rows; w: V0, mu, lambda
    uint32_t snh;
    float l0, l1;     // multipliers at the end of the previous sweep
};

__device__ __forceinline__ TetRec load_tet(const SceneDev& s, uint32_t t) {
    TetRec r;
    r.id = __ldg(&s.tet[t]);
    r.a = __ldg(&s.dm0[t]);
    r.b = __ldg(&s.dm1[t]);
    r.c = __ldg(&s.dm2[t]);
    r.snh = s.model[t] != 0;
    r.l0 = __ldcg(&s.lam0[t]);
    r.l1 = r.snh ? __ldcg(&s.lam1[t]) : 0.0f;
    return r;
}

// The part of a record the staged copies do not carry: the model flag and
// the multipliers.
__device__ __forceinline__ void load_tet_dyn(const SceneDev& s, uint32_t t, TetRec& r) {
    r.snh = s.model[t] != 0;
    r.l0 = __ldcg(&s.lam0[t]);
    r.l1 = r.snh ? __ldcg(&s.lam1[t]) : 0.0f;
}

// One elastic tet constraint (StVK: green_constraint.cpp:49-158; SNH coupled).
__device__ __forceinline__ void project_tet_rec(const SceneDev& s, const StepParams& p, uint32_t t,
                                                const TetRec& R, bool first) {
    const bool snh = R.snh != 0;
    const uint4 id = R.id;
    const float4 a = R.a, b = R.b, c = R.c;
    float4 q0 = __ldcg(&s.xi[id.x]);
    float4 q1 = __ldcg(&s.xi[id.y]);
    float4 q2 = __ldcg(&s.xi[id.z]);
    float4 q3 = __ldcg(&s.xi[id.w]);
    const float w[4] = {q0.w, q1.w, q2.w, q3.w};
    const f3 x0 = mk(q0), x1 = mk(q1), x2 = mk(q2), x3 = mk(q3);
    const f3 r0 = mk(a), r1 = mk(b), r2 = mk(c);
    f3 dx[4];
    bool moved = false;
    if (!snh) {
        TetEval e;
        stvk_eval(x0, x1, x2, x3, r0, r1, r2, a.w, b.w, c.w, e);
        const float lacc = first ? 0.0f : R.l0;
        float gd = 0.0f;
        if (p.stvk_damping) {
            // sum_i f_i . (xi_i - xn_i) with f = -g
            const float4 n0 = s.xn[id.x], n1 = s.xn[id.y], n2 = s.xn[id.z], n3 = s.xn[id.w];
            gd = -(dot(e.g[0], x0 - mk(n0)) + dot(e.g[1], x1 - mk(n1)) + dot(e.g[2], x2 - mk(n2)) +
                   dot(e.g[3], x3 - mk(n3)));
        }
        const float dl = stvk_dlambda(e, w, lacc, p.stvk_alpha_tilde, p.stvk_gamma, gd);
        s.lam0[t] = lacc + dl;
        if (dl != 0.0f) {
            moved = true;
#pragma unroll
            for (int i = 0; i < 4; ++i) dx[i] = e.g[i] * (w[i] * dl);
        }
    } else {
        float lD = first ? 0.0f : R.l0;
        float lH = first ? 0.0f : R.l1;
        float dlD, dlH;
        if (snh_step(x0, x1, x2, x3, r0, r1, r2, fabsf(a.w), b.w, c.w, p.inv_dt2, w, lD, lH, dx, dlD,
                     dlH)) {
            lD += dlD;
            lH += dlH;
            moved = true;
        }
        s.lam0[t] = lD;
        s.lam1[t] = lH;
    }
    if (moved) {
        q0.x += dx[0].x; q0.y += dx[0].y; q0.z += dx[0].z;
        q1.x += dx[1].x; q1.y += dx[1].y; q1.z += dx[1].z;
        q2.x += dx[2].x; q2.y += dx[2].y; q2.z += dx[2].z;
        q3.x += dx[3].x; q3.y += dx[3].y; q3.z += dx[3].z;
        s.xi[id.x] = q0;
        s.xi[id.y] = q1;
        s.xi[id.z] = q2;
        s.xi[id.w] = q3;
    }
}

__device__ __forceinline__ void project_tet(const SceneDev& s, const StepParams& p, uint32_t t, bool first) {
    project_tet_rec(s, p, t, load_tet(s, t), first);
}

// First tet slot of this thread in colour `col` under for_each_spread's
// mapping (chunk wib * gridDim.x + blockIdx.x, lane), or ~0u.
__device__ __forceinline__ uint32_t first_slot(const StepParams& p, int col) {
    const uint32_t b = p.colour_start[col], n = p.colour_start[col + 1] - b;
    const uint32_t c = (threadIdx.x >> 5) * gridDim.x + blockIdx.x;
    const uint32_t i = (c << 5) + (threadIdx.x & 31u);
    return i < n ? b + i : ~0u;
}

// colour_phase with the first tet's record already loaded (slot ~0u: none).
__device__ __forceinline__ void colour_phase_pf(const SceneDev& s, const StepParams& p, int col, bool first,
                                                uint32_t slot, const TetRec& rec) {
    if (slot != ~0u) project_tet_rec(s, p, slot, rec, first);
    const uint32_t lane = threadIdx.x & 31u, wpb = blockDim.x >> 5;
    const uint32_t b = p.colour_start[col], n = p.colour_start[col + 1] - b;
    const uint32_t chunks = (n + 31u) >> 5;
    for (uint32_t c = (threadIdx.x >> 5) * gridDim.x + blockIdx.x + gridDim.x * wpb; c < chunks;
         c += gridDim.x * wpb) {
        const uint32_t i = (c << 5) + lane;
        if (i < n) project_tet(s, p, b + i, first);
    }
}

__device__ __forceinline__ void colour_phase(const SceneDev& s, const StepParams& p, int col, bool first) {
    const uint32_t b = p.colour_start[col], e = p.colour_start[col + 1], m = p.colour_split[col];
    (void)m;
    for_each_spread(b, e, [&](uint32_t t) { project_tet(s, p, t, first); });
}

// Tail colours in one CTA, separated by CTA barriers.
__device__ __forceinline__ void tail_phase(const SceneDev& s, const StepParams& p, bool first) {
    for (int col = p.first_tail; col < p.n_colours; ++col) {
        const uint32_t b = p.colour_start[col], e = p.colour_start[col + 1], m = p.colour_split[col];
        (void)m;
        for (uint32_t t = b + threadIdx.x; t < e; t += blockDim.x) project_tet(s, p, t, first);
        __syncthreads();
    }
}

// distance_constraint_t::project_positions (distance_constraint.cpp:24-53).
// Coincident ends (where the reference divides by zero) and a zero
// denominator leave the constraint unchanged.
__device__ __forceinline__ void project_edge(const SceneDev& s, const StepParams& p, uint32_t k, bool first) {
    const uint2 e = s.edge[k];
    const float4 q = s.edge_p[k];
    float lam = first ? 0.0f : s.edge_lam[k];
    float4 p1 = __ldcg(&s.xi[e.x]);
    float4 p2 = __ldcg(&s.xi[e.y]);
    const float w1 = p1.w, w2 = p2.w;
    const f3 diff = mk(p1) - mk(p2);
    const float length = sqrtf(dot(diff, diff));
    if (length > 0.0f) {
        const f3 n = diff * (1.0f / length);
        const float C = length - q.x;
        const float at = q.y * p.inv_dt2;
        const float bt = q.z * p.dt * p.dt;
        const float gamma = at * bt * p.inv_dt;
        float gd = 0.0f;
        if (q.z != 0.0f) {
            const float4 n1 = s.xn[e.x], n2 = s.xn[e.y];
            gd = dot(n, mk(p1) - mk(n1)) - dot(n, mk(p2) - mk(n2));
        }
        const float den = (1.0f + gamma) * (w1 + w2) + at;
        if (den > 0.0f) {
            const float dl = (-(C + at * lam) + gamma * gd) / den;
            lam += dl;
            p1.x += w1 * n.x * dl; p1.y += w1 * n.y * dl; p1.z += w1 * n.z * dl;
            p2.x -= w2 * n.x * dl; p2.y -= w2 * n.y * dl; p2.z -= w2 * n.z * dl;
            s.xi[e.x] = p1;
            s.xi[e.y] = p2;
        }
    }
    s.edge_lam[k] = lam;
}

__device__ __forceinline__ void contact_phase(const SceneDev& s, uint32_t seg, uint32_t count,
                                              const StepParams& p, bool first) {
    for_each_spread(seg, seg + count, [&](uint32_t ci) { project_contact(s, p, ci, first); });
}

// ---------------------------------------------------------------------------
// Per-phase kernels (graph mode)

__global__ void k_edges(SceneDev s, StepParams p, int colour, int first) {
    for_each_spread(p.edge_start[colour], p.edge_start[colour + 1],
                    [&](uint32_t k) { project_edge(s, p, k, first != 0); });
}

__global__ void k_detect(SceneDev s, StepParams p) {
    const uint32_t n = s.n_surf * (uint32_t)p.n_planes;
    // whole warps stay converged for the ballot: iterate over warp-aligned ranges
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t k = base + (threadIdx.x & 31u);
        if (k < n) detect_item(s, p, k);
    }
}

__global__ void k_predict(SceneDev s, StepParams p, int substep, int has_acc) {
    // simulation time before this substep: the finalize of the previous one
    // added dt to *s.time (same double sequence as the CPU loop)
    const double t_next = *s.time + p.dt_d;
    for_each_vertex(s.n_verts, [&](uint32_t i) { predict_vertex(s, p, i, t_next, has_acc); });
}

__global__ void k_contacts(SceneDev s, StepParams p, int first) {
    for (int pl = 0; pl < p.n_planes; ++pl) {
        // planes are processed in order; a vertex may touch several planes
        const uint32_t cnt = min(s.counters[pl], s.n_surf);
        contact_phase(s, (uint32_t)pl * s.n_surf, cnt, p, first != 0);
        if (p.n_planes > 1) __syncthreads();  // single-CTA launch when several planes
    }
}

// Body-body contacts of the frame (after the ground contacts, as they follow
// them in the collision constraint list).
__global__ void k_contacts_body(SceneDev s, StepParams p, int first) {
    const uint32_t cnt = min(s.counters[kMaxPlanes], s.n_surf);
    contact_phase(s, (uint32_t)kMaxPlanes * s.n_surf, cnt, p, first != 0);
}

__global__ void k_colour(SceneDev s, StepParams p, int col, int first) { colour_phase(s, p, col, first != 0); }

__global__ void k_tail(SceneDev s, StepParams p, int first) { tail_phase(s, p, first != 0); }

__global__ void k_finalize(SceneDev s, StepParams p) {
    for_each_vertex(s.n_verts, [&](uint32_t i) { finalize_vertex(s, p, i); });
    if (blockIdx.x == 0 && threadIdx.x == 0) *s.time = *s.time + p.dt_d;
}

// End of frame: keep the frame's contact counts (for introspection) in
// counters[kMaxPlanes+1 ..] and zero the live counters for the next frame.
__global__ void k_end_frame(SceneDev s) {
    const int i = threadIdx.x;
    if (i <= kMaxPlanes) {
        s.counters[kMaxPlanes + 1 + i] = s.counters[i];
        s.counters[i] = 0;
    }
}

// ---------------------------------------------------------------------------
// Persistent frame kernel

__device__ __forceinline__ void st_release(uint32_t* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned ld_relaxed_u(const unsigned* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Wavefront wait: warp 0 polls the progress counters of this CTA's
// neighbours (relaxed loads, all of a lane's in flight at once) until each
// has finished `need` colour phases, then one acquire fence; bounded by
// s.wait_ns (then SBS_ETIMEOUT).  The CTA then passes a CTA barrier.
__device__ __forceinline__ bool wave_wait(const SceneDev& s, uint32_t need) {
    __shared__ int s_ok;
    if (threadIdx.x < 32) {
        int ok = 1;
        const uint32_t b = s.nb_start[blockIdx.x], e = s.nb_start[blockIdx.x + 1];
        const unsigned long long t0 = global_ns();
        unsigned spins = 0;
        for (;;) {
            bool mine = true;
            for (uint32_t k = b + threadIdx.x; k < e; k += 32) mine &= ld_relaxed_u(s.prog + s.nb[k]) >= need;
            if (__all_sync(0xffffffffu, mine)) break;
            if ((++spins & 15u) == 0) {
                int stop = 0;
                if (threadIdx.x == 0) {
                    if (ld_relaxed(s.err) != 0) stop = 1;
                    else if (global_ns() - t0 > s.wait_ns) {
                        atomicCAS(s.err, 0, kErrTimeout);
                        stop = 1;
                    }
                }
                if (__shfl_sync(0xffffffffu, stop, 0)) { ok = 0; break; }
            }
        }
        __threadfence();   // acquire: the neighbours' released writes are visible after this
        if (threadIdx.x == 0) s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// ---- staged tet records (persistent mode, kStage): each warp copies the
// 64-byte rest records (corner ids, DmInv rows) of the 32 tets it projects
// first in the next colour phase into its own shared-memory buffer with four
// bulk asynchronous copies completing on the warp's mbarrier, issued at the
// start of the current phase - a whole phase and grid barrier of lead
// instead of the load between the barrier's arrive and wait.  Two buffers
// per warp alternate.  Dynamic shared memory: 2 x warps x 4 x 32 x 16 bytes.
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void pmb_init(uint32_t mb) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
}

// Bounded wait for the completion of phase `parity` of an mbarrier.
__device__ __forceinline__ bool pmb_wait(uint32_t mb, uint32_t parity, unsigned long long limit_ns) {
    unsigned long long t0 = 0;
    for (uint32_t spins = 0;; ++spins) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mb), "r"(parity)
            : "memory");
        if (done) return true;
        if (spins == 0) t0 = global_ns();
        else if ((spins & 15u) == 0 && global_ns() - t0 > limit_ns) return false;
    }
}

struct WarpStage {
    uint32_t buf_base;     // shared address of this warp's two buffers
    uint32_t mb_base;      // shared address of this warp's two mbarriers
    uint32_t phase[2];     // completed (and consumed) phases of each mbarrier
    bool pending[2];       // a copy into the buffer is in flight or unconsumed
    uint32_t n[2];         // tets staged in the buffer
};

constexpr uint32_t kStageWarpBytes = 4u * 32u * 16u;   // one buffer: ids + 3 DmInv rows of 32 tets

// Lane 0 issues the copies of this warp's first chunk of colour `col` into
// buffer `buf`; every lane records whether it did.
__device__ __forceinline__ void stage_chunk(const SceneDev& s, const StepParams& p, int col, WarpStage& w,
                                            int buf) {
    const uint32_t b = p.colour_start[col], n = p.colour_start[col + 1] - b;
    const uint32_t i0 = (((threadIdx.x >> 5) * gridDim.x + blockIdx.x) << 5);
    const uint32_t cnt = i0 < n ? min(32u, n - i0) : 0u;
    w.pending[buf] = cnt > 0;
    w.n[buf] = cnt;
    if (cnt == 0) return;
    __syncwarp();   // every lane has read the buffer's previous contents
    if ((threadIdx.x & 31u) == 0) {
        const uint32_t bytes = cnt * 16u, dst = w.buf_base + (uint32_t)buf * kStageWarpBytes;
        const uint32_t mb = w.mb_base + (uint32_t)buf * 8u;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(4u * bytes) : "memory");
        const void* src[4] = {s.tet + b + i0, s.dm0 + b + i0, s.dm1 + b + i0, s.dm2 + b + i0};
#pragma unroll
        for (int k = 0; k < 4; ++k)
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                         ::"r"(dst + (uint32_t)k * 512u), "l"(src[k]), "r"(bytes), "r"(mb) : "memory");
    }
}

// Waits for buffer `buf` (false: the wait ran out, SBS_ETIMEOUT recorded).
__device__ __forceinline__ bool stage_wait(const SceneDev& s, WarpStage& w, int buf) {
    if (!w.pending[buf]) return true;
    const bool ok = pmb_wait(w.mb_base + (uint32_t)buf * 8u, w.phase[buf] & 1u, s.wait_ns);
    w.phase[buf]++;
    w.pending[buf] = false;
    if (!ok) atomicCAS(s.err, 0, kErrTimeout);
    return ok;
}

template <bool kWave, bool kStage>
__global__ void __launch_bounds__(512) k_frame_t(SceneDev s, StepParams p, int has_acc) {
    if (ld_relaxed(s.err) != 0) return;
    extern __shared__ __align__(16) uint4 stage_smem[];
    __shared__ __align__(8) unsigned long long s_pmb[2 * 16];
    WarpStage ws{};
    if (kStage) {
        const uint32_t wib = threadIdx.x >> 5;
        ws.buf_base = smem_u32(stage_smem) + wib * 2u * kStageWarpBytes;
        ws.mb_base = smem_u32(&s_pmb[2 * wib]);
        if ((threadIdx.x & 31u) == 0) {
            pmb_init(ws.mb_base);
            pmb_init(ws.mb_base + 8u);
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncwarp();
    }
    int sb = 0;                // staging buffer of the current colour phase
    // before leaving on an error: no bulk copy may still be writing into
    // this CTA's shared memory
    auto drain = [&]() {
        if (kStage) {
            stage_wait(s, ws, 0);
            stage_wait(s, ws, 1);
        }
    };
    uint32_t done = 0;         // wavefront: colour phases this CTA has finished
    unsigned bar_target = 0;   // arrivals expected by the next barrier (host zeroes s.bar[0])
    double t = *s.time;
    // contacts from frame-start positions
    {
        const uint32_t n = s.n_surf * (uint32_t)p.n_planes;
        const uint32_t stride = gridDim.x * blockDim.x;
        for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
            const uint32_t k = base + (threadIdx.x & 31u);
            if (k < n) detect_item(s, p, k);
        }
    }
    if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
    uint32_t cnt[kMaxPlanes];
    for (int pl = 0; pl < kMaxPlanes; ++pl) cnt[pl] = pl < p.n_planes ? min(__ldcg(&s.counters[pl]), s.n_surf) : 0u;
    const uint32_t cnt_body = p.body_contacts ? min(__ldcg(&s.counters[kMaxPlanes]), s.n_surf) : 0u;
    bool any_contact = cnt_body > 0;
    for (int pl = 0; pl < p.n_planes; ++pl) any_contact |= cnt[pl] > 0;
    for (int sub = 0; sub < p.substeps; ++sub) {
        const double t_next = t + p.dt_d;
        for_each_vertex(s.n_verts, [&](uint32_t i) { predict_vertex(s, p, i, t_next, has_acc); });
        if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
        for (int it = 0; it < p.iterations; ++it) {
            const bool first = it == 0;
            uint32_t slot = (!kWave && p.first_tail > 0) ? first_slot(p, 0) : ~0u;
            TetRec rec;
            if (kStage) {
                // the frame's first colour phase is staged here; later ones
                // by the phase before them
                if (sub == 0 && it == 0 && p.first_tail > 0) stage_chunk(s, p, 0, ws, sb);
                if (slot != ~0u) load_tet_dyn(s, slot, rec);
            } else if (slot != ~0u) {
                rec = load_tet(s, slot);
            }
            for (int pl = 0; pl < p.n_planes; ++pl) {
                if (cnt[pl] == 0) continue;
                contact_phase(s, (uint32_t)pl * s.n_surf, cnt[pl], p, first);
                if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
            }
            if (cnt_body) {
                contact_phase(s, (uint32_t)kMaxPlanes * s.n_surf, cnt_body, p, first);
                if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
            }
            if (kWave) {
                // every colour, each CTA its own slice; wait only for the
                // neighbours (GS order is kept: a tet of colour c runs after
                // every vertex-sharing tet of colours < c has finished, and
                // before any of colours > c starts)
                for (int col = 0; col < p.n_colours; ++col) {
                    const uint32_t* ws = s.wave_start + (size_t)col * (gridDim.x + 1) + blockIdx.x;
                    const uint32_t b = ws[0], e = ws[1];
                    const uint32_t k0 = b + threadIdx.x;
                    uint32_t t0 = 0;
                    TetRec r;
                    if (k0 < e) {
                        t0 = s.wave_idx[k0];
                        r = load_tet(s, t0);
                    }
                    if (!wave_wait(s, done)) return;
                    if (k0 < e) project_tet_rec(s, p, t0, r, first);
                    for (uint32_t k = k0 + blockDim.x; k < e; k += blockDim.x) project_tet(s, p, s.wave_idx[k], first);
                    __syncthreads();
                    ++done;
                    if (threadIdx.x == 0) st_release(s.prog + blockIdx.x, done);
                }
            } else {
            for (int col = 0; col < p.first_tail; ++col) {
                if (kStage) {
                    // the next colour phase of the frame (the next iteration's
                    // or substep's first one after the last colour)
                    const bool last = col + 1 == p.first_tail && it + 1 == p.iterations && sub + 1 == p.substeps;
                    if (!last) stage_chunk(s, p, col + 1 < p.first_tail ? col + 1 : 0, ws, sb ^ 1);
                    if (!stage_wait(s, ws, sb)) slot = ~0u;
                    if (slot != ~0u) {
                        const uint4* B = stage_smem + (threadIdx.x >> 5) * (2u * kStageWarpBytes / 16u) +
                                         (uint32_t)sb * (kStageWarpBytes / 16u);
                        const uint32_t lane = threadIdx.x & 31u;
                        rec.id = B[lane];
                        const uint4 r0 = B[32 + lane], r1 = B[64 + lane], r2 = B[96 + lane];
                        rec.a = make_float4(__uint_as_float(r0.x), __uint_as_float(r0.y), __uint_as_float(r0.z),
                                            __uint_as_float(r0.w));
                        rec.b = make_float4(__uint_as_float(r1.x), __uint_as_float(r1.y), __uint_as_float(r1.z),
                                            __uint_as_float(r1.w));
                        rec.c = make_float4(__uint_as_float(r2.x), __uint_as_float(r2.y), __uint_as_float(r2.z),
                                            __uint_as_float(r2.w));
                    }
                    sb ^= 1;
                }
                colour_phase_pf(s, p, col, first, slot, rec);
                grid_arrive(s.bar, bar_target);
                slot = col + 1 < p.first_tail ? first_slot(p, col + 1) : ~0u;
                if (slot != ~0u) {
                    if (kStage) load_tet_dyn(s, slot, rec);
                    else rec = load_tet(s, slot);
                }
                if (!grid_wait(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
            }
            }
            if (!kWave && p.first_tail < p.n_colours) {
                if (blockIdx.x == 0) tail_phase(s, p, first);
                if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
            }
            if (kWave && (p.n_edge_colours > 0 || (it + 1 < p.iterations && any_contact))) {
                // distance constraints and the next iteration's contacts touch
                // vertices of any CTA: a grid barrier before them
                if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
            }
            for (int col = 0; col < p.n_edge_colours; ++col) {
                for_each_spread(p.edge_start[col], p.edge_start[col + 1],
                                [&](uint32_t k) { project_edge(s, p, k, first); });
                if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
            }
        }
        if (kWave && !(p.n_edge_colours > 0)) {
            // the velocity update reads every vertex
            if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
        }
        for_each_vertex(s.n_verts, [&](uint32_t i) { finalize_vertex(s, p, i); });
        t = t_next;
    }
    if (!grid_barrier(s.bar, s.err, bar_target, s.wait_ns)) { drain(); return; }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        *s.time = t;
        for (int i = 0; i <= kMaxPlanes; ++i) {
            s.counters[kMaxPlanes + 1 + i] = s.counters[i];
            s.counters[i] = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// Residual and energy with compensated FP32 sums (Neumaier's variant of
// Kahan summation; pairs combined with Knuth's two-sum).


__device__ __forceinline__ CSum block_reduce(CSum v, float* sh) {
    // sh: 2 * blockDim.x floats
    sh[threadIdx.x] = v.s;
    sh[blockDim.x + threadIdx.x] = v.e;
    __syncthreads();
    for (unsigned off = blockDim.x >> 1; off > 0; off >>= 1) {
        if (threadIdx.x < off) {
            CSum a{sh[threadIdx.x], sh[blockDim.x + threadIdx.x]};
            a.merge(CSum{sh[threadIdx.x + off], sh[blockDim.x + threadIdx.x + off]});
            sh[threadIdx.x] = a.s;
            sh[blockDim.x + threadIdx.x] = a.e;
        }
        __syncthreads();
    }
    CSum r{sh[0], sh[blockDim.x]};
    __syncthreads();
    return r;
}

// zero_lam: the residual the state would have with every multiplier zero
// (the plain start of a substep: the predicted positions, nothing solved).
__global__ void k_residual(SceneDev s, StepParams p, int cnt_base, int zero_lam) {
    extern __shared__ float sh[];
    CSum re{0.f, 0.f}, en{0.f, 0.f}, rc{0.f, 0.f};
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < s.n_tets; t += stride) {
        const uint4 id = s.tet[t];
        const float4 a = s.dm0[t], b = s.dm1[t], c = s.dm2[t];
        const f3 x0 = mk(s.xi[id.x]), x1 = mk(s.xi[id.y]), x2 = mk(s.xi[id.z]), x3 = mk(s.xi[id.w]);
        const bool snh = s.model[t] != 0;
        if (!snh) {
            TetEval e;
            stvk_eval(x0, x1, x2, x3, mk(a), mk(b), mk(c), a.w, b.w, c.w, e);
            const float h = e.C + (zero_lam ? 0.0f : p.stvk_alpha_tilde * s.lam0[t]);
            re.add(h * h);
            en.add(e.C);
        } else {
            float r2, E;
            snh_residual(x0, x1, x2, x3, mk(a), mk(b), mk(c), fabsf(a.w), b.w, c.w, p.inv_dt2,
                         zero_lam ? 0.0f : s.lam0[t], zero_lam ? 0.0f : s.lam1[t], r2, E);
            re.add(r2);
            en.add(E);
        }
    }
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < s.n_edges; k += stride) {
        const uint2 e = s.edge[k];
        const float4 q = s.edge_p[k];
        const f3 d = mk(s.xi[e.x]) - mk(s.xi[e.y]);
        const float C = sqrtf(dot(d, d)) - q.x;
        const float h = C + (zero_lam ? 0.0f : q.y * p.inv_dt2 * s.edge_lam[k]);
        re.add(h * h);
        if (q.y > 0.0f) en.add(0.5f * C * C / q.y);
    }
    for (int pl = 0; pl <= kMaxPlanes; ++pl) {
        // planes, then the body-contact segment (index kMaxPlanes)
        if (pl < kMaxPlanes && pl >= p.n_planes) continue;
        const uint32_t cnt = min(s.counters[cnt_base + pl], s.n_surf);
        for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < cnt; k += stride) {
            const uint32_t ci = (uint32_t)pl * s.n_surf + k;
            const Contact c = s.contacts[ci];
            const float4 x = s.xi[__float_as_uint(c.q.w)];
            const float C = (x.x - c.q.x) * c.n.x + (x.y - c.q.y) * c.n.y + (x.z - c.q.z) * c.n.z;
            if (C < 0.0f) {
                const float h = C + (zero_lam ? 0.0f : p.contact_alpha_tilde * s.contact_lam[ci]);
                rc.add(h * h);
            }
        }
    }
    re = block_reduce(re, sh);
    en = block_reduce(en, sh);
    rc = block_reduce(rc, sh);
    if (threadIdx.x == 0) {
        float* o = s.partials + 6 * blockIdx.x;
        o[0] = re.s; o[1] = re.e; o[2] = en.s; o[3] = en.e; o[4] = rc.s; o[5] = rc.e;
    }
}

// Sums the per-CTA partials (fixed order) into red_out and, for a judged
// warm-started substep, acts on the residual r = sqrt(elastic^2 + contact^2)
// (JudgeOp): records the plain start's residual, decides between the warm
// and the plain start and whether the sweep loop runs, counts a chunk of
// sweeps and decides whether another one runs, or records a plain substep's
// residual as the target.  The loop decision goes to the loop's conditional
// graph node; it is 0 once the residual is at or below the target, the next
// chunk would pass the sweep cap, or the device error flag is set, so the
// loop always ends.
__global__ void k_residual_final(SceneDev s, int nparts, JudgeOp op) {
    extern __shared__ float sh[];
    CSum acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    for (int i = threadIdx.x; i < nparts; i += blockDim.x)
        for (int k = 0; k < 3; ++k) acc[k].merge(CSum{s.partials[6 * i + 2 * k], s.partials[6 * i + 2 * k + 1]});
    double red[3];
    for (int k = 0; k < 3; ++k) {
        CSum r = block_reduce(acc[k], sh);
        red[k] = (double)r.s + (double)r.e;
        if (threadIdx.x == 0) s.red_out[k] = red[k];
    }
    if (threadIdx.x != 0 || op.kind == kJudgeNone) return;
    JudgeDev* j = op.j;
    const double sq = red[0] + red[2];
    const double r = sq > 0.0 ? sqrt(sq) : (sq == sq ? 0.0 : sq);   // NaN stays NaN
    const double target = j->target[op.substep];
    const bool err = *(volatile int*)s.err != 0;
    unsigned cond = 0;
    switch (op.kind) {
    case kJudgePlain0:
        j->r_plain0 = r;
        return;
    case kJudgeStart: {
        // a start whose residual is not below the plain start's is discarded
        const bool fb = !(r < j->r_plain0);
        j->fallback = fb ? 1u : 0u;
        if (fb) j->fallbacks++;
        j->r_start = fb ? j->r_plain0 : r;
        j->r_now = j->r_start;
        j->sweeps = 0;
        cond = (!(j->r_now <= target) && op.chunk <= op.cap && !err) ? 1u : 0u;
        break;
    }
    case kJudgeChunk:
        j->sweeps += op.chunk;
        j->r_now = r;
        cond = (!(r <= target) && j->sweeps + op.chunk <= op.cap && !err) ? 1u : 0u;
        break;
    case kJudgeCalib:
        j->target[op.substep] = r;
        j->calib_substeps++;
        return;
    default:
        return;
    }
    cudaGraphSetConditional((cudaGraphConditionalHandle)op.cond, cond);
}

__global__ void k_set_error(int* err, int code) { atomicCAS(err, 0, code); }

// ---------------------------------------------------------------------------
// Launchers

static inline int grid_for(uint32_t n, int block, int cap) {
    long g = ((long)n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (int)g;
}

cudaError_t launch_detect_ground(const SceneDev& s, const StepParams& p, cudaStream_t st) {
    const uint32_t n = s.n_surf * (uint32_t)p.n_planes;
    if (n == 0) return cudaSuccess;
    k_detect<<<grid_for(n, 256, 4096), 256, 0, st>>>(s, p);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_edges(const SceneDev& s, const StepParams& p, int colour, int first_iter, cudaStream_t st) {
    const uint32_t n = p.edge_start[colour + 1] - p.edge_start[colour];
    if (n == 0) return cudaSuccess;
    k_edges<<<grid_for((n + 31) / 32 * 32, 256, 1024), 256, 0, st>>>(s, p, colour, first_iter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_predict(const SceneDev& s, const StepParams& p, int substep, cudaStream_t st) {
    (void)substep;
    k_predict<<<grid_for(s.n_verts, 256, 8192), 256, 0, st>>>(s, p, substep, p.has_acc);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_contacts(const SceneDev& s, const StepParams& p, int first_iter, cudaStream_t st) {
    if (p.n_planes == 0 || s.n_surf == 0) return cudaSuccess;
    const int grid = p.n_planes > 1 ? 1 : grid_for(s.n_surf, 256, 1024);
    k_contacts<<<grid, 256, 0, st>>>(s, p, first_iter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_body_contacts(const SceneDev& s, const StepParams& p, int first_iter, cudaStream_t st) {
    if (!p.body_contacts || s.n_surf == 0) return cudaSuccess;
    k_contacts_body<<<grid_for(s.n_surf, 256, 1024), 256, 0, st>>>(s, p, first_iter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_colour(const SceneDev& s, const StepParams& p, int colour, int first_iter, int block,
                          int grid, cudaStream_t st) {
    k_colour<<<grid, block, 0, st>>>(s, p, colour, first_iter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_tail(const SceneDev& s, const StepParams& p, int first_iter, int block, cudaStream_t st) {
    if (p.first_tail >= p.n_colours) return cudaSuccess;
    k_tail<<<1, block, 0, st>>>(s, p, first_iter);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_finalize(const SceneDev& s, const StepParams& p, cudaStream_t st) {
    k_finalize<<<grid_for(s.n_verts, 256, 8192), 256, 0, st>>>(s, p);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    return cudaSuccess;
}

cudaError_t launch_end_frame(const SceneDev& s, cudaStream_t st) {
    k_end_frame<<<1, 32, 0, st>>>(s);
    count_launch();
    return cudaGetLastError();
}

cudaError_t launch_residual_ex(const SceneDev& s, const StepParams& p, int block, int grid, int cnt_base,
                               cudaStream_t st, int zero_lam, const JudgeOp* op) {
    const size_t shm = 2 * sizeof(float) * (size_t)block;
    k_residual<<<grid, block, shm, st>>>(s, p, cnt_base, zero_lam);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    JudgeOp none{};
    none.kind = kJudgeNone;
    k_residual_final<<<1, 256, 2 * sizeof(float) * 256, st>>>(s, grid, op ? *op : none);
    count_launch();
    return cudaGetLastError();
}

static size_t stage_bytes(int block) { return (size_t)(block / 32) * 2u * kStageWarpBytes; }

cudaError_t persistent_occupancy(int block, int* ctas_per_sm, int stage) {
    if (stage) {
        cudaError_t e = cudaFuncSetAttribute(k_frame_t<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)stage_bytes(512));
        if (e != cudaSuccess) return e;
        return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, k_frame_t<false, true>, block,
                                                             stage_bytes(block));
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, k_frame_t<false, false>, block, 0);
}

cudaError_t wavefront_occupancy(int block, int* ctas_per_sm) {
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas_per_sm, k_frame_t<true, false>, block, 0);
}

cudaError_t launch_wavefront_frame(const SceneDev& s, const StepParams& p, int block, int grid, cudaStream_t st) {
    int has_acc = p.has_acc;
    SceneDev sc = s;
    StepParams pc = p;
    void* args[] = {&sc, &pc, &has_acc};
    count_launch();
    return cudaLaunchCooperativeKernel((const void*)k_frame_t<true, false>, dim3(grid), dim3(block), args, 0, st);
}

cudaError_t launch_persistent_frame(const SceneDev& s, const StepParams& p, int block, int grid,
                                    cudaStream_t st, int stage) {
    int has_acc = p.has_acc;
    SceneDev sc = s;
    StepParams pc = p;
    void* args[] = {&sc, &pc, &has_acc};
    count_launch();
    if (stage)
        return cudaLaunchCooperativeKernel((const void*)k_frame_t<false, true>, dim3(grid), dim3(block), args,
                                           stage_bytes(block), st);
    return cudaLaunchCooperativeKernel((const void*)k_frame_t<false, false>, dim3(grid), dim3(block), args, 0, st);
}

cudaError_t launch_set_error(int* err, int code, cudaStream_t st) {
    k_set_error<<<1, 1, 0, st>>>(err, code);
    count_launch();
    return cudaGetLastError();
}

}  // namespace sbs
