// Cluster-resident XPBD frame kernel for sm_103a.
//
// A thread-block cluster of C CTAs (C <= 16) owns a group of whole bodies.
// The group's vertex state (xi, xn, v) is split into C contiguous slices,
// one per CTA, and kept in shared memory for the whole frame; tets gather
// and scatter their four vertices through distributed shared memory
// (mapa + ld/st.shared::cluster).  Colour phases are separated by the
// hardware cluster barrier (barrier.cluster.arrive.release / wait.acquire),
// so a frame needs no grid-wide synchronisation at all and clusters working
// on different groups never wait for one another.
//
// The sweep is the same Gauss-Seidel order as the global kernels: per
// iteration the group's contacts (each touches one vertex; a vertex's planes
// in plane order), then the colours one after another (timestep.cpp:20-70,
// gauss_seidel_solver.cpp:8-37).
//
// With the learned warm start a launch runs one substep instead
// (StepParams::cl_flags): the global kernels predict and warm-start the
// positions, the kernel takes them and the carried multipliers from global
// memory, sweeps, and writes both back; the frame's contacts come from the
// global contact list.
#include <cuda_runtime.h>
#include <stdint.h>

#include "cluster_internal.cuh"
#include "launch_count.cuh"
#include "xpbd_internal.cuh"
#include "xpbd_math.cuh"

namespace sbs {

__device__ __forceinline__ uint32_t cl_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cl_id() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ uint32_t cl_count() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync() {
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
// the two halves of cluster_sync, for work between a CTA's arrival and the
// barrier's completion
__device__ __forceinline__ void cluster_arrive() {
    __syncwarp();
    asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory");
}
__device__ __forceinline__ void cluster_wait() {
    __syncwarp();
    asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint32_t map_rank(uint32_t addr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
    return r;
}
__device__ __forceinline__ float4 ld_dsmem(uint32_t addr) {
    float4 v;
    asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_dsmem_u32(uint32_t addr) {
    uint32_t v;
    asm volatile("ld.shared::cluster.u32 %0, [%1];" : "=r"(v) : "r"(addr) : "memory");
    return v;
}
__device__ __forceinline__ void st_dsmem(uint32_t addr, float4 v) {
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};"
                 :: "r"(addr), "f"(v.x), "f"(v.y), "f"(v.z), "f"(v.w) : "memory");
}

// Address of packed vertex (rank << 24 | local) in the cluster's xi slices.
__device__ __forceinline__ uint32_t vaddr(uint32_t packed, uint32_t xi_base) {
    return map_rank(xi_base + ((packed & 0xFFFFFFu) << 4), (packed >> 24) & 0x7Fu);
}

// The read-only part of a tet's record: the DSMEM addresses of its corners'
// xi and its rest data.  (Loading the next colour's record into registers
// across the cluster barrier was measured slower: 6.9 against 6.3 ms per
// frame of the 98k-tet beam; the records are staged in shared memory by
// bulk copies instead, see k_cluster_frame.)
struct ClTet {
    uint32_t a0, a1, a2, a3;
    float4 a, b, c;   // DmInv rows; w: V0, mu, lambda
    uint32_t snh;
};

__device__ __forceinline__ ClTet cl_make_tet(uint4 id, float4 a, float4 b, float4 c, uint32_t xi_base) {
    ClTet r;
    r.a0 = vaddr(id.x, xi_base);
    r.a1 = vaddr(id.y, xi_base);
    r.a2 = vaddr(id.z, xi_base);
    r.a3 = vaddr(id.w, xi_base);
    r.a = a;
    r.b = b;
    r.c = c;
    r.snh = id.x >> 31;
    return r;
}

__device__ __forceinline__ ClTet cl_load_tet(const SceneDev& s, const ClusterDev& c, uint32_t t, uint32_t xi_base) {
    return cl_make_tet(__ldg(&c.tet_packed[t]), __ldg(&s.dm0[t]), __ldg(&s.dm1[t]), __ldg(&s.dm2[t]), xi_base);
}

// ---- staging of tet records: bulk asynchronous copies (TMA) completing on an
// mbarrier.  Thread 0 issues a colour phase's copies at the start of the
// phase before it; the threads that read the records wait on the mbarrier.
// (Other arrangements measured slower on the 98k-tet beam: the wait by one
// thread or a producer warp before the barrier, two phases of lead with three
// buffers, per-thread cp.async copies.)
constexpr int kErrTimeoutCl = 3;   // SBS_ETIMEOUT

__device__ __forceinline__ unsigned long long cl_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mb_init(uint32_t mb) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mb) : "memory");
}
__device__ __forceinline__ void mb_arrive_tx(uint32_t mb, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mb_arrive(uint32_t mb) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mb) : "memory");
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mb) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 ::"r"(dst), "l"(src), "r"(bytes), "r"(mb) : "memory");
}
// Bounded wait for phase `parity` of the mbarrier; false after limit_ns
// (SceneDev::wait_ns).  One probe inline; the timed loop out of line, so the
// colour-phase loop carries only the probe.
__device__ __noinline__ bool mb_wait_slow(uint32_t mb, uint32_t parity, unsigned long long limit_ns) {
    const unsigned long long t0 = cl_ns();
    for (uint32_t spins = 1;; ++spins) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(mb), "r"(parity)
            : "memory");
        if (done) return true;
        if ((spins & 15u) == 0 && cl_ns() - t0 > limit_ns) return false;
    }
}

__device__ __forceinline__ bool mb_wait(uint32_t mb, uint32_t parity, unsigned long long limit_ns) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(mb), "r"(parity)
        : "memory");
    return done ? true : mb_wait_slow(mb, parity, limit_ns);
}

// Stage the records of tets [b, e) (at most c.stage) into buffer `buf`:
// packed ids, then the three DmInv rows, each an array of c.stage float4.
// Elements are 16 bytes, so every source and destination is 16-byte aligned.
__device__ __forceinline__ void stage_issue(const SceneDev& s, const ClusterDev& c, uint32_t b, uint32_t e,
                                            uint32_t buf_addr, uint32_t mb) {
    const uint32_t n = e - b;
    if (n == 0) {
        mb_arrive(mb);
        return;
    }
    const uint32_t bytes = n * 16u, arr = c.stage * 16u;
    mb_arrive_tx(mb, 4u * bytes);
    bulk_g2s(buf_addr, c.tet_packed + b, bytes, mb);
    bulk_g2s(buf_addr + arr, s.dm0 + b, bytes, mb);
    bulk_g2s(buf_addr + 2u * arr, s.dm1 + b, bytes, mb);
    bulk_g2s(buf_addr + 3u * arr, s.dm2 + b, bytes, mb);
}

// lam: this tet's multipliers in the CTA's shared memory (lam[0]; SNH's
// hydrostatic one at lam[lstride]).
__device__ __forceinline__ void project_tet_dsmem(const ClusterDev& c, const StepParams& p, const ClTet& T,
                                                  bool first, float* lam, uint32_t lstride) {
    const bool snh = T.snh != 0;
    const float4 a = T.a, b = T.b, cc = T.c;
    const uint32_t a0 = T.a0, a1 = T.a1, a2 = T.a2, a3 = T.a3;
    float4 q0 = ld_dsmem(a0), q1 = ld_dsmem(a1), q2 = ld_dsmem(a2), q3 = ld_dsmem(a3);
    const float w[4] = {q0.w, q1.w, q2.w, q3.w};
    const f3 x0 = mk(q0), x1 = mk(q1), x2 = mk(q2), x3 = mk(q3);
    const f3 r0 = mk(a), r1 = mk(b), r2 = mk(cc);
    f3 dx[4];
    bool moved = false;
    if (!snh) {
        TetEval e;
        stvk_eval(x0, x1, x2, x3, r0, r1, r2, a.w, b.w, cc.w, e);
        const float lacc = first ? 0.0f : lam[0];
        float gd = 0.0f;
        if (p.stvk_damping) {
            // xn of the tet's vertices: the global copy holds the frame-start
            // state only, so damping uses the per-slice xn (same packed ids)
            const float4 n0 = ld_dsmem(a0 + c.xn_minus_xi), n1 = ld_dsmem(a1 + c.xn_minus_xi),
                         n2 = ld_dsmem(a2 + c.xn_minus_xi), n3 = ld_dsmem(a3 + c.xn_minus_xi);
            gd = -(dot(e.g[0], x0 - mk(n0)) + dot(e.g[1], x1 - mk(n1)) + dot(e.g[2], x2 - mk(n2)) +
                   dot(e.g[3], x3 - mk(n3)));
        }
        const float dl = stvk_dlambda(e, w, lacc, p.stvk_alpha_tilde, p.stvk_gamma, gd);
        lam[0] = lacc + dl;
        if (dl != 0.0f) {
            moved = true;
#pragma unroll
            for (int i = 0; i < 4; ++i) dx[i] = e.g[i] * (w[i] * dl);
        }
    } else {
        float lD = first ? 0.0f : lam[0];
        float lH = first ? 0.0f : lam[lstride];
        float dlD, dlH;
        if (snh_step(x0, x1, x2, x3, r0, r1, r2, fabsf(a.w), b.w, cc.w, p.inv_dt2, w, lD, lH, dx, dlD, dlH)) {
            lD += dlD;
            lH += dlH;
            moved = true;
        }
        lam[0] = lD;
        lam[lstride] = lH;
    }
    if (moved) {
        q0.x += dx[0].x; q0.y += dx[0].y; q0.z += dx[0].z;
        q1.x += dx[1].x; q1.y += dx[1].y; q1.z += dx[1].z;
        q2.x += dx[2].x; q2.y += dx[2].y; q2.z += dx[2].z;
        q3.x += dx[3].x; q3.y += dx[3].y; q3.z += dx[3].z;
        st_dsmem(a0, q0);
        st_dsmem(a1, q1);
        st_dsmem(a2, q2);
        st_dsmem(a3, q3);
    }
}

// ---- plain-solver judge inside the kernel (kClJudge) ----
// Residual of the group's constraints, sqrt(sum (C + alpha~ lambda)^2) over
// the tets and the contacts, at the positions in the cluster's slices and the
// multipliers in shared memory: each CTA sums its own tets and contact
// vertices (compensated FP32; per thread, then per warp by shuffles, then
// the warps in order), publishes (sum, error, flag) in its shared memory, and
// after a cluster barrier every CTA adds the CTAs' partials in rank order, so
// every CTA gets the same value and takes the same loop decision.  `flag`
// carries a CTA's view of the device error flag (a staging wait that ran
// out), made cluster-uniform the same way; the result is then NaN.
struct ClPart {
    float s, e, flag, pad;
};

__device__ __forceinline__ float cl_tet_res2(const ClTet& T, const StepParams& p, float l0, float l1) {
    const float4 q0 = ld_dsmem(T.a0), q1 = ld_dsmem(T.a1), q2 = ld_dsmem(T.a2), q3 = ld_dsmem(T.a3);
    const f3 x0 = mk(q0), x1 = mk(q1), x2 = mk(q2), x3 = mk(q3);
    if (T.snh) {
        float r2, E;
        snh_residual(x0, x1, x2, x3, mk(T.a), mk(T.b), mk(T.c), fabsf(T.a.w), T.b.w, T.c.w, p.inv_dt2, l0, l1, r2,
                     E);
        return r2;
    }
    TetEval e;
    stvk_eval(x0, x1, x2, x3, mk(T.a), mk(T.b), mk(T.c), T.a.w, T.b.w, T.c.w, e);
    const float h = e.C + p.stvk_alpha_tilde * l0;
    return h * h;
}

__device__ __forceinline__ double cl_residual(const SceneDev& s, const ClusterDev& c, const StepParams& p,
                                              uint32_t n_col, const uint32_t* cb, const uint32_t* ce,
                                              const uint32_t* lbase, const float* lam_s, const uint32_t* clist,
                                              uint32_t ncont, const float4* xi, const float4* rec, const float4* bn,
                                              int S, uint32_t xi_base, bool bad, ClPart* part, CSum* warp_sum,
                                              double* out) {
    CSum acc{0.f, 0.f};
    for (uint32_t col = 0; col < n_col; ++col) {
        const uint32_t b = cb[col], e = ce[col];
        const float* lb = lam_s + lbase[col] - b;
        for (uint32_t tt = b + threadIdx.x; tt < e; tt += blockDim.x)
            acc.add(cl_tet_res2(cl_load_tet(s, c, tt, xi_base), p, lb[tt], lb[tt + c.lcap]));
    }
    for (uint32_t k = threadIdx.x; k < ncont; k += blockDim.x) {
        const uint32_t i = clist[k];
        const float4 x = xi[i];
        for (int sl = 0; sl < S; ++sl) {
            const float4 r = rec[(size_t)i * S + sl];
            if (isnan(r.x)) continue;
            float nx, ny, nz;
            if (sl < p.n_planes) {
                nx = p.planes[sl].nx; ny = p.planes[sl].ny; nz = p.planes[sl].nz;
            } else {
                const float4 nn = bn[i];
                nx = nn.x; ny = nn.y; nz = nn.z;
            }
            const float C_ = (x.x - r.x) * nx + (x.y - r.y) * ny + (x.z - r.z) * nz;
            if (C_ < 0.0f) {
                const float h = C_ + p.contact_alpha_tilde * r.w;
                acc.add(h * h);
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        CSum o{__shfl_down_sync(0xffffffffu, acc.s, off), __shfl_down_sync(0xffffffffu, acc.e, off)};
        acc.merge(o);
    }
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    if (lane == 0) warp_sum[wid] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        CSum t = warp_sum[0];
        for (uint32_t w = 1; w < (blockDim.x + 31) / 32; ++w) t.merge(warp_sum[w]);
        const bool b = bad || *(volatile int*)s.err != 0;
        *part = ClPart{t.s, t.e, b ? 1.0f : 0.0f, 0.0f};
    }
    cluster_sync();
    if (threadIdx.x == 0) {
        const uint32_t a = smem_addr(part);
        CSum t{0.f, 0.f};
        bool any_bad = false;
        for (uint32_t r = 0; r < c.cluster_size; ++r) {
            const float4 q = ld_dsmem(map_rank(a, r));
            t.merge(CSum{q.x, q.y});
            any_bad |= q.z != 0.0f;
        }
        const double sq = (double)t.s + (double)t.e;
        *out = any_bad ? __longlong_as_double(0x7ff8000000000000ll) : (sq > 0.0 ? sqrt(sq) : 0.0);
    }
    __syncthreads();
    return *out;
}

// Shared memory per CTA: two staging buffers for the tet records of one
// colour phase (4 * c.stage float4 each: packed ids, DmInv rows; filled one
// phase ahead while the current phase projects), xi[slice], xn[slice],
// v[slice] (float4 each),
// contact records rec[slice * n_planes] (q.xyz, lambda; q.x = NaN when the
// vertex has no contact with that plane), their slots in the global contact
// list gidx[slice * n_planes], and the CTA's contact vertex list clist[slice].
// The plain frame: the whole frame of a group per launch (prediction,
// sweeps, velocity update), or one warm-started substep with the
// kClExternal / kClCarry / kClContinue flags.  Kept apart from the judge's
// kernel below so that the hot loop of plain frames carries none of its code
// (measured: sharing one templated body made the 98k-tet beam's frame 4-5%
// slower).
__global__ void __launch_bounds__(kClusterMaxBlock) k_cluster_frame_plain(SceneDev s, ClusterDev c, StepParams p,
                                                                           double t0) {
    extern __shared__ float4 sm[];
    const uint32_t rank = cl_rank();
    const uint32_t C = c.cluster_size;
    const uint32_t slice = c.slice;
    const float4* stg = sm;                        // 2 staging buffers of 4 * c.stage float4
    float4* xi = sm + 8 * (size_t)c.stage;
    float4* xn = xi + slice;
    float4* vv = xi + 2 * slice;
    const int S = p.n_planes + (c.body ? 1 : 0);   // contact slots per vertex: planes, then body
    float4* rec = xi + 3 * slice;
    float4* bn = rec + (size_t)slice * S;          // body contact normals (when c.body)
    uint32_t* gidx = reinterpret_cast<uint32_t*>(bn + (c.body ? slice : 0));
    uint32_t* clist = gidx + (size_t)slice * S;
    float* lam_s = reinterpret_cast<float*>(clist + slice);   // [2 * lcap] multipliers of this CTA's tets
    __shared__ uint32_t s_ncont;
    __shared__ uint32_t s_any_contact;
    // this CTA's tet range and multiplier base per colour of the current
    // group, kept on chip: they head every colour phase's dependency chain
    __shared__ uint32_t s_cb[kMaxColours], s_ce[kMaxColours], s_lb[kMaxColours];
    __shared__ __align__(8) unsigned long long s_mb[2];   // one mbarrier per staging buffer
    const uint32_t xi_base = smem_addr(xi);
    const uint32_t stg_base = smem_addr(stg), stg_bytes = c.stage * 64u, mb_base = smem_addr(s_mb);
    // colour phases run so far (all groups): staging buffer ph & 1, whose
    // mbarrier is then in its (ph >> 1)-th phase
    uint32_t ph = 0;
    bool stage_bad = false;   // a staging wait expired: this thread projects nothing more
    ClTet nrec{};             // this thread's first record of the next colour phase, when have_next
    bool have_next = false;
    if (c.stage && threadIdx.x == 0) {
        mb_init(mb_base);
        mb_init(mb_base + 8);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    for (uint32_t g = cl_id(); g < c.n_groups; g += cl_count()) {
        const GroupDesc gd = c.groups[g];
        const uint32_t own0 = gd.v0 + rank * slice;
        const uint32_t own1 = min(gd.v0 + (rank + 1) * slice, gd.v0 + gd.nv);
        const uint32_t nown = own1 > own0 ? own1 - own0 : 0;
        if (threadIdx.x == 0) s_ncont = 0;
        for (uint32_t col = threadIdx.x; col < gd.n_col; col += blockDim.x) {
            const uint32_t k = gd.col_base + col * C + rank;
            s_cb[col] = c.col_start[k];
            s_ce[col] = c.col_start[k + 1];
            s_lb[col] = c.lam_base[gd.lb_base + col * C + rank];
        }
        __syncthreads();
        // the group's first colour phase: its records arrive while the slice loads
        if (c.stage && threadIdx.x == 0 && gd.n_col > 0 && p.substeps > 0 && p.iterations > 0)
            stage_issue(s, c, s_cb[0], s_ce[0], stg_base + (ph & 1u) * stg_bytes, mb_base + (ph & 1u) * 8u);
        const bool ext = (p.cl_flags & kClExternal) != 0;
        // load own slice; ground contacts of own surface vertices from the
        // frame-start positions (bvh_model.cpp:72-94 with the plane SDF)
        for (uint32_t i = threadIdx.x; i < nown && ext; i += blockDim.x) {
            // one warm-started substep: positions as predicted and moved by
            // the warm start; contacts from the frame's list (below)
            const uint32_t gv = own0 + i;
            xi[i] = s.xi[gv];
            xn[i] = s.xn[gv];
            vv[i] = s.v[gv];
            for (int pl = 0; pl < p.n_planes; ++pl)
                rec[(size_t)i * S + pl] = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
            if (c.body) {
                const float4 bq = c.bc_q[gv];
                float4 r = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
                if (bq.w != 0.0f) {
                    const float4 nn = c.bc_n[gv];
                    r = make_float4(bq.x, bq.y, bq.z, 0.0f);
                    bn[i] = nn;
                    gidx[(size_t)i * S + p.n_planes] = __float_as_uint(nn.w);
                }
                rec[(size_t)i * S + p.n_planes] = r;
            }
        }
        if (ext) {
            __syncthreads();
            for (int pl = 0; pl < p.n_planes; ++pl) {
                const uint32_t cnt = min(__ldcg(&s.counters[pl]), s.n_surf);
                for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
                    const Contact ct = s.contacts[(size_t)pl * s.n_surf + k];
                    const uint32_t gv = __float_as_uint(ct.q.w);
                    if (gv < own0 || gv >= own1) continue;
                    const uint32_t i = gv - own0;
                    rec[(size_t)i * S + pl] = make_float4(ct.q.x, ct.q.y, ct.q.z, 0.0f);
                    gidx[(size_t)i * S + pl] = k;
                }
            }
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) {
                bool any = false;
                for (int sl = 0; sl < S; ++sl) any |= !isnan(rec[(size_t)i * S + sl].x);
                if (any) clist[atomicAdd(&s_ncont, 1u)] = i;
            }
            if (p.cl_flags & kClCarry) {
                // the multipliers the warm start left (carried or fitted)
                for (uint32_t col = 0; col < gd.n_col; ++col) {
                    const uint32_t b = s_cb[col], e = s_ce[col];
                    float* lb = lam_s + s_lb[col] - b;
                    for (uint32_t tt = b + threadIdx.x; tt < e; tt += blockDim.x) {
                        lb[tt] = s.lam0[tt];
                        lb[tt + c.lcap] = s.lam1[tt];
                    }
                }
            }
        }
        for (uint32_t i = threadIdx.x; i < nown && !ext; i += blockDim.x) {
            const uint32_t gv = own0 + i;
            const float4 x = s.xn[gv];
            xn[i] = x;
            xi[i] = x;
            vv[i] = s.v[gv];
            bool any = false;
            const bool surf = (c.vflags[gv] & 1u) != 0;
            for (int pl = 0; pl < p.n_planes; ++pl) {
                const Plane P = p.planes[pl];
                const float sd = P.nx * x.x + P.ny * x.y + P.nz * x.z + P.d;
                float4 r = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
                if (surf && sd < 0.0f) {
                    const float ad = fabsf(sd);
                    r = make_float4(x.x + P.nx * ad, x.y + P.ny * ad, x.z + P.nz * ad, 0.0f);
                    any = true;
                    // publish in the frame's global contact list (introspection, residual)
                    const uint32_t slot = atomicAdd(&s.counters[pl], 1u);
                    gidx[(size_t)i * S + pl] = slot;
                    if (slot < s.n_surf) {
                        Contact ct;
                        ct.q = make_float4(r.x, r.y, r.z, __uint_as_float(gv));
                        ct.n = make_float4(P.nx, P.ny, P.nz, 0.0f);
                        s.contacts[(size_t)pl * s.n_surf + slot] = ct;
                    }
                }
                rec[(size_t)i * S + pl] = r;
            }
            if (c.body) {
                // body-body contact found by the spatial hash for this vertex
                const float4 bq = c.bc_q[gv];
                float4 r = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
                if (bq.w != 0.0f) {
                    const float4 nn = c.bc_n[gv];
                    r = make_float4(bq.x, bq.y, bq.z, 0.0f);
                    bn[i] = nn;
                    gidx[(size_t)i * S + p.n_planes] = __float_as_uint(nn.w);
                    any = true;
                }
                rec[(size_t)i * S + p.n_planes] = r;
            }
            if (any) clist[atomicAdd(&s_ncont, 1u)] = i;
        }
        cluster_sync();
        const uint32_t ncont = s_ncont;
        // does any CTA of the cluster hold a contact this frame?  (the same
        // answer everywhere, so the contact phase and its barrier are skipped
        // cluster-wide when none does)
        if (threadIdx.x == 0) {
            uint32_t any = 0;
            for (uint32_t r = 0; r < C; ++r) any |= ld_dsmem_u32(map_rank(smem_addr(&s_ncont), r));
            s_any_contact = any;
        }
        __syncthreads();
        const bool group_contacts = s_any_contact != 0;
        double t = t0;
        for (int sub = 0; sub < p.substeps; ++sub) {
            const double t_next = t + p.dt_d;
            // prediction of own vertices (timestep.cpp:35-43) + prescribed motion
            for (uint32_t i = threadIdx.x; i < nown && !ext; i += blockDim.x) {
                float4 v = vv[i];
                const float4 x = xn[i];
                if (v.w != 0.0f) {
                    const KinGroup k = p.kin[(int)v.w - 1];
                    const float4 rel = s.acc[own0 + i];
                    float sn, cs;
                    sincosf((float)(k.omega * t_next), &sn, &cs);
                    const f3 ax = mk(k.ax, k.ay, k.az), r = mk(rel.x, rel.y, rel.z);
                    const f3 rr = r * cs + cross(ax, r) * sn + ax * (dot(ax, r) * (1.0f - cs));
                    xi[i] = make_float4(k.cx + rr.x, k.cy + rr.y, k.cz + rr.z, x.w);
                    continue;
                }
                const float w = x.w;
                float ax = 0.f, ay = 0.f, az = 0.f;
                if (w > 0.0f) {
                    if (p.gravity_mode == 1) { ax = p.gx * w; ay = p.gy * w; az = p.gz * w; }
                    else { ax = p.gx; ay = p.gy; az = p.gz; }
                    if (p.has_acc) {
                        const float4 e = s.acc[own0 + i];
                        ax += e.x; ay += e.y; az += e.z;
                    }
                }
                v.x += ax * p.dt;
                v.y += ay * p.dt;
                v.z += az * p.dt;
                vv[i] = v;
                xi[i] = make_float4(x.x + v.x * p.dt, x.y + v.y * p.dt, x.z + v.z * p.dt, w);
            }
            cluster_sync();
            for (int it = 0; it < p.iterations; ++it) {
                const bool first = it == 0;                                 // contacts start from 0
                const bool first_lam = first && !(p.cl_flags & kClCarry);  // elastic multipliers
                // contacts: own vertices only (collision_constraint.cpp:21-41)
                for (uint32_t k = threadIdx.x; k < ncont; k += blockDim.x) {
                    const uint32_t i = clist[k];
                    float4 x = xi[i];
                    for (int sl = 0; sl < S; ++sl) {
                        float4 r = rec[(size_t)i * S + sl];
                        if (isnan(r.x)) continue;
                        if (first) r.w = 0.0f;
                        float nx, ny, nz;
                        if (sl < p.n_planes) {
                            nx = p.planes[sl].nx; ny = p.planes[sl].ny; nz = p.planes[sl].nz;
                        } else {
                            const float4 nn = bn[i];
                            nx = nn.x; ny = nn.y; nz = nn.z;
                        }
                        const float C_ = (x.x - r.x) * nx + (x.y - r.y) * ny + (x.z - r.z) * nz;
                        if (C_ < 0.0f) {
                            const float w = x.w;
                            const float dl = -(C_ + p.contact_alpha_tilde * r.w) / (w + p.contact_alpha_tilde);
                            r.w += dl;
                            x.x += w * nx * dl;
                            x.y += w * ny * dl;
                            x.z += w * nz * dl;
                        }
                        rec[(size_t)i * S + sl] = r;
                    }
                    xi[i] = x;
                }
                if (S > 0 && group_contacts) cluster_sync();  // cluster-uniform condition
                for (uint32_t col = 0; col < gd.n_col; ++col) {
                    // this CTA's tets of the colour: those owning most of their vertices here
                    const uint32_t b = s_cb[col], e = s_ce[col];
                    float* lb = lam_s + s_lb[col] - b;
                    // the frame's next colour phase: the next colour, or the
                    // next iteration's or substep's first one after the last
                    const bool last_phase = sub + 1 == p.substeps && it + 1 == p.iterations && col + 1 == gd.n_col;
                    const uint32_t nc = col + 1 == gd.n_col ? 0u : col + 1;
                    if (c.stage) {
                        const uint32_t buf = ph & 1u;
                        if (threadIdx.x == 0 && !last_phase) {
                            // next phase's records into the other buffer, whose
                            // readers all passed the cluster barrier behind us
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            stage_issue(s, c, s_cb[nc], s_ce[nc], stg_base + (buf ^ 1u) * stg_bytes,
                                        mb_base + (buf ^ 1u) * 8u);
                        }
                        if (b + threadIdx.x < e && !stage_bad) {
                            // the first record came in during the last barrier (have_next)
                            if (have_next || mb_wait(mb_base + buf * 8u, (ph >> 1) & 1u, s.wait_ns)) {
                                const float4* B = stg + (size_t)buf * 4 * c.stage;
                                const uint4* I = reinterpret_cast<const uint4*>(B);
                                const uint32_t k0 = threadIdx.x;
                                project_tet_dsmem(c, p,
                                                  have_next ? nrec
                                                            : cl_make_tet(I[k0], B[c.stage + k0], B[2 * c.stage + k0],
                                                                          B[3 * c.stage + k0], xi_base),
                                                  first_lam, lb + b + k0, c.lcap);
                                for (uint32_t k = k0 + blockDim.x; k < e - b; k += blockDim.x)
                                    project_tet_dsmem(c, p,
                                                      cl_make_tet(I[k], B[c.stage + k], B[2 * c.stage + k],
                                                                  B[3 * c.stage + k], xi_base),
                                                      first_lam, lb + b + k, c.lcap);
                            } else {
                                stage_bad = true;
                                atomicCAS(s.err, 0, kErrTimeoutCl);
                            }
                        }
                        ++ph;
                        // arrive, then take this thread's first record of the next
                        // phase out of its staging buffer while the other CTAs
                        // arrive: the wait for the copy and the shared-memory loads
                        // leave the head of the next phase
                        cluster_arrive();
                        have_next = false;
                        if (!last_phase && !stage_bad && s_cb[nc] + threadIdx.x < s_ce[nc]) {
                            const uint32_t nbuf = ph & 1u;
                            if (mb_wait(mb_base + nbuf * 8u, (ph >> 1) & 1u, s.wait_ns)) {
                                const float4* B = stg + (size_t)nbuf * 4 * c.stage;
                                const uint4* I = reinterpret_cast<const uint4*>(B);
                                const uint32_t k0 = threadIdx.x;
                                nrec = cl_make_tet(I[k0], B[c.stage + k0], B[2 * c.stage + k0], B[3 * c.stage + k0],
                                                   xi_base);
                                have_next = true;
                            } else {
                                stage_bad = true;
                                atomicCAS(s.err, 0, kErrTimeoutCl);
                            }
                        }
                        cluster_wait();
                    } else {
                        for (uint32_t tt = b + threadIdx.x; tt < e; tt += blockDim.x)
                            project_tet_dsmem(c, p, cl_load_tet(s, c, tt, xi_base), first_lam, lb + tt, c.lcap);
                        cluster_sync();
                    }
                }
            }
            // velocity update of own vertices (timestep.cpp:48-57)
            for (uint32_t i = threadIdx.x; i < nown && !ext; i += blockDim.x) {
                const float4 a = xi[i];
                const float4 b = xn[i];
                float4 v = vv[i];
                v.x = (a.x - b.x) * p.inv_dt;
                v.y = (a.y - b.y) * p.inv_dt;
                v.z = (a.z - b.z) * p.inv_dt;
                vv[i] = v;
                xn[i] = a;
            }
            t = t_next;
            __syncthreads();
        }
        // write back the slice and the multipliers of the last substep
        for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) {
            const uint32_t gv = own0 + i;
            s.xi[gv] = xi[i];
            s.xn[gv] = xn[i];
            s.v[gv] = vv[i];
        }
        for (uint32_t col = 0; col < gd.n_col; ++col) {
            const uint32_t k = gd.col_base + col * C + rank;
            const uint32_t b = c.col_start[k], e = c.col_start[k + 1];
            const float* lb = lam_s + c.lam_base[gd.lb_base + col * C + rank] - b;
            for (uint32_t tt = b + threadIdx.x; tt < e; tt += blockDim.x) {
                s.lam0[tt] = lb[tt];
                s.lam1[tt] = lb[tt + c.lcap];
            }
        }
        for (uint32_t k = threadIdx.x; k < ncont; k += blockDim.x) {
            const uint32_t i = clist[k];
            for (int sl = 0; sl < S; ++sl) {
                const float4 r = rec[(size_t)i * S + sl];
                const uint32_t slot = gidx[(size_t)i * S + sl];
                const size_t seg = sl < p.n_planes ? (size_t)sl : (size_t)kMaxPlanes;
                if (!isnan(r.x) && slot < s.n_surf) s.contact_lam[seg * s.n_surf + slot] = r.w;
            }
        }
        __syncthreads();
    }
    // no CTA may leave while a peer could still read its shared memory
    cluster_sync();
}

// MODE: kClModeJudge (judged warm-started substeps, kClJudge),
// kClModeCalib (calibration frames, kClCalibrate) or kClModePlain (further
// chunks of a judged substep's sweeps in the global judge loop,
// kClContinue).
constexpr int kClModePlain = 0, kClModeJudge = 1, kClModeCalib = 2;
template <int MODE>
__global__ void __launch_bounds__(kClusterMaxBlock) k_cluster_frame(SceneDev s, ClusterDev c, StepParams p,
                                                                     double t0) {
    extern __shared__ float4 sm[];
    const uint32_t rank = cl_rank();
    const uint32_t C = c.cluster_size;
    const uint32_t slice = c.slice;
    const float4* stg = sm;                        // 2 staging buffers of 4 * c.stage float4
    float4* xi = sm + 8 * (size_t)c.stage;
    float4* xn = xi + slice;
    float4* vv = xi + 2 * slice;
    const int S = p.n_planes + (c.body ? 1 : 0);   // contact slots per vertex: planes, then body
    float4* rec = xi + 3 * slice;
    float4* bn = rec + (size_t)slice * S;          // body contact normals (when c.body)
    uint32_t* gidx = reinterpret_cast<uint32_t*>(bn + (c.body ? slice : 0));
    uint32_t* clist = gidx + (size_t)slice * S;
    float* lam_s = reinterpret_cast<float*>(clist + slice);   // [2 * lcap] multipliers of this CTA's tets
    __shared__ uint32_t s_ncont;
    __shared__ uint32_t s_any_contact;
    // this CTA's tet range and multiplier base per colour of the current
    // group, kept on chip: they head every colour phase's dependency chain
    __shared__ uint32_t s_cb[kMaxColours], s_ce[kMaxColours], s_lb[kMaxColours];
    __shared__ __align__(8) unsigned long long s_mb[2];   // one mbarrier per staging buffer
    __shared__ __align__(16) ClPart s_part;               // the judge's residual partial of this CTA
    __shared__ CSum s_wsum[kClusterMaxBlock / 32];
    __shared__ double s_res;
    const uint32_t xi_base = smem_addr(xi);
    const uint32_t stg_base = smem_addr(stg), stg_bytes = c.stage * 64u, mb_base = smem_addr(s_mb);
    // colour phases run so far (all groups): staging buffer ph & 1, whose
    // mbarrier is then in its (ph >> 1)-th phase
    uint32_t ph = 0;
    bool stage_bad = false;   // a staging wait expired: this thread projects nothing more
    if (c.stage && threadIdx.x == 0) {
        mb_init(mb_base);
        mb_init(mb_base + 8);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    for (uint32_t g = cl_id(); g < c.n_groups; g += cl_count()) {
        const GroupDesc gd = c.groups[g];
        const uint32_t own0 = gd.v0 + rank * slice;
        const uint32_t own1 = min(gd.v0 + (rank + 1) * slice, gd.v0 + gd.nv);
        const uint32_t nown = own1 > own0 ? own1 - own0 : 0;
        if (threadIdx.x == 0) s_ncont = 0;
        for (uint32_t col = threadIdx.x; col < gd.n_col; col += blockDim.x) {
            const uint32_t k = gd.col_base + col * C + rank;
            s_cb[col] = c.col_start[k];
            s_ce[col] = c.col_start[k + 1];
            s_lb[col] = c.lam_base[gd.lb_base + col * C + rank];
        }
        __syncthreads();
        // the group's first colour phase: its records arrive while the slice loads
        // (judged substeps issue it at the start of each chunk of sweeps instead)
        // a judged substep (kClJudge), or a calibration frame (kClCalibrate):
        // plain substeps that record their final residuals as the targets
        constexpr bool calib = MODE == kClModeCalib;
        constexpr bool judged = MODE == kClModeJudge;
        if (c.stage && threadIdx.x == 0 && gd.n_col > 0 && p.substeps > 0 && p.iterations > 0 && !judged)
            stage_issue(s, c, s_cb[0], s_ce[0], stg_base + (ph & 1u) * stg_bytes, mb_base + (ph & 1u) * 8u);
        const bool ext = (p.cl_flags & kClExternal) != 0;
        // a further chunk of the same substep's sweeps: the contact
        // multipliers go on from where the previous chunk left them
        const bool cont = ext && (p.cl_flags & kClContinue) != 0;
        // load own slice; ground contacts of own surface vertices from the
        // frame-start positions (bvh_model.cpp:72-94 with the plane SDF)
        for (uint32_t i = threadIdx.x; i < nown && ext; i += blockDim.x) {
            // one warm-started substep: positions as predicted and moved by
            // the warm start; contacts from the frame's list (below)
            const uint32_t gv = own0 + i;
            xi[i] = s.xi[gv];
            xn[i] = s.xn[gv];
            vv[i] = s.v[gv];
            for (int pl = 0; pl < p.n_planes; ++pl)
                rec[(size_t)i * S + pl] = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
            if (c.body) {
                const float4 bq = c.bc_q[gv];
                float4 r = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
                if (bq.w != 0.0f) {
                    const float4 nn = c.bc_n[gv];
                    const uint32_t slot = __float_as_uint(nn.w);
                    const float l = (cont && slot < s.n_surf) ? s.contact_lam[(size_t)kMaxPlanes * s.n_surf + slot]
                                                              : 0.0f;
                    r = make_float4(bq.x, bq.y, bq.z, l);
                    bn[i] = nn;
                    gidx[(size_t)i * S + p.n_planes] = slot;
                }
                rec[(size_t)i * S + p.n_planes] = r;
            }
        }
        if (ext) {
            __syncthreads();
            for (int pl = 0; pl < p.n_planes; ++pl) {
                const uint32_t cnt = min(__ldcg(&s.counters[pl]), s.n_surf);
                for (uint32_t k = threadIdx.x; k < cnt; k += blockDim.x) {
                    const Contact ct = s.contacts[(size_t)pl * s.n_surf + k];
                    const uint32_t gv = __float_as_uint(ct.q.w);
                    if (gv < own0 || gv >= own1) continue;
                    const uint32_t i = gv - own0;
                    const float l = cont ? s.contact_lam[(size_t)pl * s.n_surf + k] : 0.0f;
                    rec[(size_t)i * S + pl] = make_float4(ct.q.x, ct.q.y, ct.q.z, l);
                    gidx[(size_t)i * S + pl] = k;
                }
            }
            __syncthreads();
            for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) {
                bool any = false;
                for (int sl = 0; sl < S; ++sl) any |= !isnan(rec[(size_t)i * S + sl].x);
                if (any) clist[atomicAdd(&s_ncont, 1u)] = i;
            }
            if (p.cl_flags & kClCarry) {
                // the multipliers the warm start left (carried or fitted)
                for (uint32_t col = 0; col < gd.n_col; ++col) {
                    const uint32_t b = s_cb[col], e = s_ce[col];
                    float* lb = lam_s + s_lb[col] - b;
                    for (uint32_t tt = b + threadIdx.x; tt < e; tt += blockDim.x) {
                        lb[tt] = s.lam0[tt];
                        lb[tt + c.lcap] = s.lam1[tt];
                    }
                }
            }
        }
        for (uint32_t i = threadIdx.x; i < nown && !ext; i += blockDim.x) {
            const uint32_t gv = own0 + i;
            const float4 x = s.xn[gv];
            xn[i] = x;
            xi[i] = x;
            vv[i] = s.v[gv];
            bool any = false;
            const bool surf = (c.vflags[gv] & 1u) != 0;
            for (int pl = 0; pl < p.n_planes; ++pl) {
                const Plane P = p.planes[pl];
                const float sd = P.nx * x.x + P.ny * x.y + P.nz * x.z + P.d;
                float4 r = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
                if (surf && sd < 0.0f) {
                    const float ad = fabsf(sd);
                    r = make_float4(x.x + P.nx * ad, x.y + P.ny * ad, x.z + P.nz * ad, 0.0f);
                    any = true;
                    // publish in the frame's global contact list (introspection, residual)
                    const uint32_t slot = atomicAdd(&s.counters[pl], 1u);
                    gidx[(size_t)i * S + pl] = slot;
                    if (slot < s.n_surf) {
                        Contact ct;
                        ct.q = make_float4(r.x, r.y, r.z, __uint_as_float(gv));
                        ct.n = make_float4(P.nx, P.ny, P.nz, 0.0f);
                        s.contacts[(size_t)pl * s.n_surf + slot] = ct;
                    }
                }
                rec[(size_t)i * S + pl] = r;
            }
            if (c.body) {
                // body-body contact found by the spatial hash for this vertex
                const float4 bq = c.bc_q[gv];
                float4 r = make_float4(__int_as_float(0x7fc00000), 0.f, 0.f, 0.f);
                if (bq.w != 0.0f) {
                    const float4 nn = c.bc_n[gv];
                    r = make_float4(bq.x, bq.y, bq.z, 0.0f);
                    bn[i] = nn;
                    gidx[(size_t)i * S + p.n_planes] = __float_as_uint(nn.w);
                    any = true;
                }
                rec[(size_t)i * S + p.n_planes] = r;
            }
            if (any) clist[atomicAdd(&s_ncont, 1u)] = i;
        }
        cluster_sync();
        const uint32_t ncont = s_ncont;
        // does any CTA of the cluster hold a contact this frame?  (the same
        // answer everywhere, so the contact phase and its barrier are skipped
        // cluster-wide when none does)
        if (threadIdx.x == 0) {
            uint32_t any = 0;
            for (uint32_t r = 0; r < C; ++r) any |= ld_dsmem_u32(map_rank(smem_addr(&s_ncont), r));
            s_any_contact = any;
        }
        __syncthreads();
        const bool group_contacts = s_any_contact != 0;
        double t = t0;
        for (int sub = 0; sub < p.substeps; ++sub) {
            const double t_next = t + p.dt_d;
            // prediction of own vertices (timestep.cpp:35-43) + prescribed motion
            for (uint32_t i = threadIdx.x; i < nown && !ext; i += blockDim.x) {
                float4 v = vv[i];
                const float4 x = xn[i];
                if (v.w != 0.0f) {
                    const KinGroup k = p.kin[(int)v.w - 1];
                    const float4 rel = s.acc[own0 + i];
                    float sn, cs;
                    sincosf((float)(k.omega * t_next), &sn, &cs);
                    const f3 ax = mk(k.ax, k.ay, k.az), r = mk(rel.x, rel.y, rel.z);
                    const f3 rr = r * cs + cross(ax, r) * sn + ax * (dot(ax, r) * (1.0f - cs));
                    xi[i] = make_float4(k.cx + rr.x, k.cy + rr.y, k.cz + rr.z, x.w);
                    continue;
                }
                const float w = x.w;
                float ax = 0.f, ay = 0.f, az = 0.f;
                if (w > 0.0f) {
                    if (p.gravity_mode == 1) { ax = p.gx * w; ay = p.gy * w; az = p.gz * w; }
                    else { ax = p.gx; ay = p.gy; az = p.gz; }
                    if (p.has_acc) {
                        const float4 e = s.acc[own0 + i];
                        ax += e.x; ay += e.y; az += e.z;
                    }
                }
                v.x += ax * p.dt;
                v.y += ay * p.dt;
                v.z += az * p.dt;
                vv[i] = v;
                xi[i] = make_float4(x.x + v.x * p.dt, x.y + v.y * p.dt, x.z + v.z * p.dt, w);
            }
            if (calib) {
                // the prediction, for the next warm substep's previous-displacement feature
                for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) p.judge_xpred[own0 + i] = xi[i];
            }
            cluster_sync();
            // Sweeps: p.iterations of them, or under the judge chunks of
            // judge_chunk until the residual reaches the target.
            const uint32_t chunk = judged ? p.judge_chunk : 1u;
            bool go = chunk > 0;
            uint32_t done = 0;       // sweeps run in this substep
            bool fb = false;
            double r_now = 0.0, target = 0.0;
            if (judged) {
                target = p.judge->target[p.judge_substep];
                const double r_plain0 = p.judge->r_plain0;
                const double r_warm = cl_residual(s, c, p, gd.n_col, s_cb, s_ce, s_lb, lam_s, clist, ncont, xi, rec,
                                                  bn, S, xi_base, stage_bad, &s_part, s_wsum, &s_res);
                // a warm start not below the plain start's residual is discarded
                fb = !(r_warm < r_plain0);
                if (fb) {
                    for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) xi[i] = p.judge_xpred[own0 + i];
                    for (uint32_t col = 0; col < gd.n_col; ++col) {
                        const uint32_t b = s_cb[col], e = s_ce[col];
                        float* lb = lam_s + s_lb[col] - b;
                        for (uint32_t tt = b + threadIdx.x; tt < e; tt += blockDim.x) {
                            lb[tt] = 0.0f;
                            lb[tt + c.lcap] = 0.0f;
                        }
                    }
                    cluster_sync();
                }
                r_now = fb ? r_plain0 : r_warm;
                go = !(r_now <= target) && chunk <= p.judge_cap;
            }
            for (int it = 0; judged ? go : it < p.iterations; ++it) {
                const uint32_t kin = judged ? (uint32_t)it % chunk : 0u;   // sweep within the chunk
                if (judged && kin == 0 && c.stage && threadIdx.x == 0 && gd.n_col > 0) {
                    // the chunk's first colour phase: its records into the buffer
                    // whose readers all passed a cluster barrier behind us
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    stage_issue(s, c, s_cb[0], s_ce[0], stg_base + (ph & 1u) * stg_bytes, mb_base + (ph & 1u) * 8u);
                }
                const bool first = it == 0;                                 // contacts start from 0
                const bool first_lam = first && !(p.cl_flags & kClCarry);  // elastic multipliers
                // contacts: own vertices only (collision_constraint.cpp:21-41)
                for (uint32_t k = threadIdx.x; k < ncont; k += blockDim.x) {
                    const uint32_t i = clist[k];
                    float4 x = xi[i];
                    for (int sl = 0; sl < S; ++sl) {
                        float4 r = rec[(size_t)i * S + sl];
                        if (isnan(r.x)) continue;
                        if (first && !cont) r.w = 0.0f;
                        float nx, ny, nz;
                        if (sl < p.n_planes) {
                            nx = p.planes[sl].nx; ny = p.planes[sl].ny; nz = p.planes[sl].nz;
                        } else {
                            const float4 nn = bn[i];
                            nx = nn.x; ny = nn.y; nz = nn.z;
                        }
                        const float C_ = (x.x - r.x) * nx + (x.y - r.y) * ny + (x.z - r.z) * nz;
                        if (C_ < 0.0f) {
                            const float w = x.w;
                            const float dl = -(C_ + p.contact_alpha_tilde * r.w) / (w + p.contact_alpha_tilde);
                            r.w += dl;
                            x.x += w * nx * dl;
                            x.y += w * ny * dl;
                            x.z += w * nz * dl;
                        }
                        rec[(size_t)i * S + sl] = r;
                    }
                    xi[i] = x;
                }
                if (S > 0 && group_contacts) cluster_sync();  // cluster-uniform condition
                for (uint32_t col = 0; col < gd.n_col; ++col) {
                    // this CTA's tets of the colour: those owning most of their vertices here
                    const uint32_t b = s_cb[col], e = s_ce[col];
                    float* lb = lam_s + s_lb[col] - b;
                    if (c.stage) {
                        const uint32_t buf = ph & 1u;
                        const bool last_phase = judged ? (kin + 1 == chunk && col + 1 == gd.n_col)
                                                       : (sub + 1 == p.substeps && it + 1 == p.iterations &&
                                                          col + 1 == gd.n_col);
                        if (threadIdx.x == 0 && !last_phase) {
                            // next phase's records into the other buffer, whose
                            // readers all passed the cluster barrier behind us
                            const uint32_t nc = col + 1 == gd.n_col ? 0u : col + 1;
                            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                            stage_issue(s, c, s_cb[nc], s_ce[nc], stg_base + (buf ^ 1u) * stg_bytes,
                                        mb_base + (buf ^ 1u) * 8u);
                        }
                        if (b + threadIdx.x < e && !stage_bad) {
                            if (mb_wait(mb_base + buf * 8u, (ph >> 1) & 1u, s.wait_ns)) {
                                const float4* B = stg + (size_t)buf * 4 * c.stage;
                                const uint4* I = reinterpret_cast<const uint4*>(B);
                                for (uint32_t k = threadIdx.x; k < e - b; k += blockDim.x)
                                    project_tet_dsmem(c, p,
                                                      cl_make_tet(I[k], B[c.stage + k], B[2 * c.stage + k],
                                                                  B[3 * c.stage + k], xi_base),
                                                      first_lam, lb + b + k, c.lcap);
                            } else {
                                stage_bad = true;
                                atomicCAS(s.err, 0, kErrTimeoutCl);
                            }
                        }
                        ++ph;
                    } else {
                        for (uint32_t tt = b + threadIdx.x; tt < e; tt += blockDim.x)
                            project_tet_dsmem(c, p, cl_load_tet(s, c, tt, xi_base), first_lam, lb + tt, c.lcap);
                    }
                    cluster_sync();
                }
                if (judged && kin + 1 == chunk) {
                    done += chunk;
                    r_now = cl_residual(s, c, p, gd.n_col, s_cb, s_ce, s_lb, lam_s, clist, ncont, xi, rec, bn, S,
                                        xi_base, stage_bad, &s_part, s_wsum, &s_res);
                    go = !(r_now <= target) && done + chunk <= p.judge_cap && !isnan(r_now);
                }
            }
            if (calib) {
                const double r = cl_residual(s, c, p, gd.n_col, s_cb, s_ce, s_lb, lam_s, clist, ncont, xi, rec, bn, S,
                                             xi_base, stage_bad, &s_part, s_wsum, &s_res);
                if (rank == 0 && threadIdx.x == 0) {
                    p.judge->target[sub < kMaxJudgeSubsteps ? sub : kMaxJudgeSubsteps - 1] = r;
                    p.judge->calib_substeps++;
                }
            }
            if (judged && rank == 0 && threadIdx.x == 0) {
                // the judge's totals (as k_judge_end), and the substep's record
                JudgeDev* j = p.judge;
                j->fallback = fb ? 1u : 0u;
                if (fb) j->fallbacks++;
                j->sweeps = done;
                j->r_now = r_now;
                j->warm_substeps++;
                j->total_sweeps += done;
                if (!(r_now <= target)) j->capped++;
                const double ratio = target > 0.0 ? r_now / target : (r_now > 0.0 ? 1e30 : 1.0);
                j->sum_ratio += ratio;
                if (ratio > j->max_ratio) j->max_ratio = ratio;
            }
            // velocity update of own vertices (timestep.cpp:48-57)
            for (uint32_t i = threadIdx.x; i < nown && !ext; i += blockDim.x) {
                const float4 a = xi[i];
                const float4 b = xn[i];
                float4 v = vv[i];
                v.x = (a.x - b.x) * p.inv_dt;
                v.y = (a.y - b.y) * p.inv_dt;
                v.z = (a.z - b.z) * p.inv_dt;
                vv[i] = v;
                xn[i] = a;
            }
            t = t_next;
            __syncthreads();
        }
        // write back the slice and the multipliers of the last substep
        for (uint32_t i = threadIdx.x; i < nown; i += blockDim.x) {
            const uint32_t gv = own0 + i;
            s.xi[gv] = xi[i];
            s.xn[gv] = xn[i];
            s.v[gv] = vv[i];
        }
        for (uint32_t col = 0; col < gd.n_col; ++col) {
            const uint32_t k = gd.col_base + col * C + rank;
            const uint32_t b = c.col_start[k], e = c.col_start[k + 1];
            const float* lb = lam_s + c.lam_base[gd.lb_base + col * C + rank] - b;
            for (uint32_t tt = b + threadIdx.x; tt < e; tt += blockDim.x) {
                s.lam0[tt] = lb[tt];
                s.lam1[tt] = lb[tt + c.lcap];
            }
        }
        for (uint32_t k = threadIdx.x; k < ncont; k += blockDim.x) {
            const uint32_t i = clist[k];
            for (int sl = 0; sl < S; ++sl) {
                const float4 r = rec[(size_t)i * S + sl];
                const uint32_t slot = gidx[(size_t)i * S + sl];
                const size_t seg = sl < p.n_planes ? (size_t)sl : (size_t)kMaxPlanes;
                if (!isnan(r.x) && slot < s.n_surf) s.contact_lam[seg * s.n_surf + slot] = r.w;
            }
        }
        __syncthreads();
    }
    // no CTA may leave while a peer could still read its shared memory
    cluster_sync();
}

// The dynamic shared-memory limit is a per-function attribute shared by every
// handle of the process, so it is raised to the most the device allows next
// to the kernel's static shared memory rather than to this scene's need: a
// later handle needing less must not make an earlier handle's launch invalid
// (measured: no change in the frame time).
template <typename K>
static cudaError_t cluster_configure_one(K kernel, size_t smem) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    if (e != cudaSuccess) return e;
    int dev = 0, optin = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, kernel)) != cudaSuccess) return e;
    const size_t max_dyn = (size_t)optin > fa.sharedSizeBytes ? (size_t)optin - fa.sharedSizeBytes : 0;
    if (smem > max_dyn) return cudaErrorInvalidValue;
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_dyn);
}

cudaError_t cluster_configure(int block, size_t smem) {
    (void)block;
    cudaError_t e = cluster_configure_one(k_cluster_frame_plain, smem);
    if (e == cudaSuccess) e = cluster_configure_one(k_cluster_frame<kClModePlain>, smem);
    if (e == cudaSuccess) e = cluster_configure_one(k_cluster_frame<kClModeJudge>, smem);
    if (e == cudaSuccess) e = cluster_configure_one(k_cluster_frame<kClModeCalib>, smem);
    return e;
}

cudaError_t cluster_max_active(int cluster_size, int block, size_t smem, int* n) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cluster_size);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = cluster_size;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaOccupancyMaxActiveClusters(n, (void*)k_cluster_frame_plain, &cfg);
}

cudaError_t launch_cluster_frame(const SceneDev& s, const ClusterDev& c, const StepParams& p, double t0,
                                 int n_clusters, int block, size_t smem, cudaStream_t st) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(n_clusters * c.cluster_size);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = c.cluster_size;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    count_launch();
    if (p.cl_flags & kClJudge) return cudaLaunchKernelEx(&cfg, k_cluster_frame<kClModeJudge>, s, c, p, t0);
    if (p.cl_flags & kClCalibrate) return cudaLaunchKernelEx(&cfg, k_cluster_frame<kClModeCalib>, s, c, p, t0);
    // a further chunk of a substep's sweeps (contact multipliers carried
    // over, kClContinue) runs the general body, every other plain launch the
    // lean one
    if (p.cl_flags & kClContinue) return cudaLaunchKernelEx(&cfg, k_cluster_frame<kClModePlain>, s, c, p, t0);
    return cudaLaunchKernelEx(&cfg, k_cluster_frame_plain, s, c, p, t0);
}

__global__ void k_store_time(double* t, double v) { *t = v; }

cudaError_t launch_store_time(double* t, double v, cudaStream_t st) {
    k_store_time<<<1, 1, 0, st>>>(t, v);
    count_launch();
    return cudaGetLastError();
}

}  // namespace sbs
