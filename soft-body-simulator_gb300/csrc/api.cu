// C ABI of the GB300 XPBD solver: scene set-up on the host (Morton order,
// boundary extraction, graph colouring), device upload, frame execution as a
// CUDA graph of per-phase kernels or as one persistent cooperative kernel,
// and state transfer.  Declarations and reference mapping: include/sbs_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/sbs_gpu.h"
#include "xpbd_internal.cuh"
#include "cluster_internal.cuh"
#include "hash_internal.cuh"
#include "mlp_internal.cuh"
#include "launch_count.cuh"
#include "surface_internal.cuh"
#include "warmstart_internal.cuh"

using namespace sbs;

namespace {

struct BodyHost {
    uint32_t v0 = 0, nv = 0, t0 = 0, nt = 0;
    std::vector<uint32_t> new_to_old;  // body-local
    std::vector<uint32_t> old_to_new;
};

struct GraphKey {
    double dt;
    uint32_t substeps, iterations;
    // 0: plain frame; warm-started frame: 1 without, 2 with the previous
    // substep's displacement known at its start; 3: a judge's calibration
    // frame (plain substeps that record their residuals as targets)
    int warm;
    bool operator<(const GraphKey& o) const {
        if (dt != o.dt) return dt < o.dt;
        if (substeps != o.substeps) return substeps < o.substeps;
        if (iterations != o.iterations) return iterations < o.iterations;
        return warm < o.warm;
    }
};

}  // namespace

struct sbs_gpu {
    sbs_gpu_params prm{};
    cudaStream_t st = nullptr;
    bool finalized = false;
    int n_sm = 0;
    std::string last_error;

    // scene as added (global "old" vertex ids = body offset + local id)
    std::vector<double> x0, xinit, mass;
    std::vector<float> vinit;            // initial velocities, 3 per vertex
    std::vector<uint8_t> user_mass;
    std::vector<uint32_t> tets;          // 4 per tet, old global ids
    std::vector<int32_t> tet_model;
    std::vector<int32_t> tet_hint;       // caller's colour per tet, -1 none (sbs_gpu_set_tet_colours)
    std::vector<double> tet_mu, tet_lam, tet_density;
    std::vector<BodyHost> bodies;
    std::vector<int32_t> kin_group;      // per old vertex, -1 free
    std::vector<KinGroup> groups;
    std::vector<float> acc;
    bool has_acc = false;
    std::vector<Plane> planes;
    // signed-distance grids of environment bodies (after the planes)
    struct GridHost {
        std::vector<float> v;
        int cubic = 0;
        uint32_t n[3];
        double o[3], h[3];
    };
    std::vector<GridHost> grids;
    std::vector<float*> grid_dev;

    // after finalize
    uint32_t n_verts = 0, n_tets = 0;
    std::vector<uint32_t> tet_order;     // slot -> global tet id
    std::vector<uint32_t> colour_offsets;
    std::vector<uint32_t> surf;          // library vertex ids
    std::vector<float> inv_mass;         // library order
    std::vector<uint8_t> is_kin;         // library order
    uint32_t n_colours = 0, first_tail = 0;
    SceneDev d{};
    StepParams base{};
    int* d_err = nullptr;
    int exec_mode = SBS_EXEC_GRAPH;
    int block = 256, grid = 0;
    int pers_block = 256, pers_grid = 0;
    int wave_grid = 0;                 // CTAs of the wavefront mode (0: unavailable)
    uint32_t wave_max_nb = 0;          // largest neighbour list
    uint32_t cl_phase_max = 0;         // cluster mode: most tets one CTA projects in one colour
    bool tuned = false;
    bool contacts_live = false;
    std::map<GraphKey, cudaGraphExec_t> graphs;
    std::map<GraphKey, uint64_t> graph_kernels;   // kernel nodes of each graph
    uint64_t kernel_launches = 0;                 // kernels run by frames since finalize
    BodyHost all_bodies;                          // the whole scene as one range (state transfer)
    uint32_t* d_o2n = nullptr;                    // global input vertex id -> library slot
    float* d_stage_x = nullptr;                   // [3V] transfer staging (positions)
    float* d_stage_v = nullptr;                   // [3V] transfer staging (velocities)
    int* d_bad = nullptr;                         // non-finite flag of a transfer
    // distance constraints: ends as global input vertex ids, parameters
    std::vector<uint32_t> dist_v;                 // 2 per constraint
    std::vector<float4> dist_p;                   // rest length, alpha, beta, 0
    std::vector<uint32_t> edge_order, edge_offsets;   // colour-major projection order
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void*> allocations;
    // cluster-resident mode
    bool cl_feasible = false, global_modes = true;
    int cl_size = 1, cl_block = 256, cl_grid = 1;
    size_t cl_smem = 0;
    uint32_t cl_slice = 1, cl_lcap = 1;
    std::vector<std::pair<uint32_t, uint32_t>> cl_groups;  // body ranges
    ClusterDev cd{};
    // body-body contacts
    bool body_on = false;
    HashDev hd{};
    double hash_cell = 0.0;
    std::vector<uint8_t> bmask;        // boundary faces per tet slot
    // learned warm start
    sbs_mlp* mlp = nullptr;
    WarmDev wd{};
    bool warm_buffers = false;
    bool xpred_valid = false;   // wd.xpred belongs to the substep that produced the current x
    // visual models, numbered as tetrahedral_mesh_boundary_t numbers them
    std::vector<uint32_t> vis_tri0, vis_sv0;   // per body + end: first triangle / surface vertex
    std::vector<uint32_t> vis_tris;            // 3 per triangle, surface-local vertex ids
    std::vector<uint32_t> vis_map;             // surface vertex -> body-local vertex id
    SurfaceDev sd{};
    uint32_t fit_sweeps = 1;
    // plain-solver judge of warm-started substeps (judge_chunk 0: off)
    uint32_t judge_chunk = 0, judge_cap = 0, judge_calib_every = 0;
    double judge_fixed_target = 0.0;
    JudgeDev* d_judge = nullptr;
    cudaStream_t side = nullptr;      // captures the bodies of the sweep loops
    uint64_t judged_frames = 0;       // judged frames run (calibration ones included)
    bool judge_target_valid = false;
    bool withhold_arrival = false;    // sbs_gpu_withhold_barrier_arrival: next persistent frame
    double sim_time = 0.0;   // host mirror of the simulation time
    std::vector<uint32_t> seg_split;  // first SNH slot of each colour segment

    // stats
    uint64_t frames = 0, projections = 0;
    double last_frame_ms = 0, residual = 0, energy = 0;
};

static thread_local std::string g_err;

static sbs_status fail(sbs_gpu* h, sbs_status s, const std::string& msg) {
    if (h) h->last_error = msg;
    g_err = msg;
    return s;
}

#define CU(h, call)                                                                        \
    do {                                                                                   \
        cudaError_t _e = (call);                                                           \
        if (_e != cudaSuccess)                                                             \
            return fail((h), SBS_ECUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    } while (0)

template <typename T>
static sbs_status dalloc(sbs_gpu* h, T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) return fail(h, SBS_ENOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    h->allocations.push_back((void*)*p);
    return SBS_OK;
}

static uint32_t expand_bits(uint32_t v) {
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// 30-bit Morton code of p inside [lo, hi].
static uint32_t morton(const double* p, const double* lo, const double* hi) {
    uint32_t c[3];
    for (int k = 0; k < 3; ++k) {
        double ext = hi[k] - lo[k];
        double u = ext > 0 ? (p[k] - lo[k]) / ext : 0.0;
        int q = (int)std::floor(u * 1023.0 + 0.5);
        c[k] = (uint32_t)std::min(1023, std::max(0, q));
    }
    return (expand_bits(c[0]) << 2) | (expand_bits(c[1]) << 1) | expand_bits(c[2]);
}

static void invert3(const double m[3][3], double r[3][3], double* det) {
    double d = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
               m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    *det = d;
    r[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) / d;
    r[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) / d;
    r[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) / d;
    r[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) / d;
    r[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) / d;
    r[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) / d;
    r[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) / d;
    r[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) / d;
    r[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) / d;
}

// Moves tets of classes above `cap` into the smallest class they fit (no
// shared vertex), visiting the tets in `order`.  When K classes cannot hold
// T tets at `cap`, empty classes are added first (K' = ceil(T / cap)) for the
// moves to fill.  A tet that fits nowhere stays.  Returns the class count.
static int balance_classes(const std::vector<uint32_t>& tets, uint32_t n_verts, const std::vector<uint32_t>& order,
                           std::vector<int32_t>& colour, int K, uint32_t cap) {
    const size_t T = order.size();
    if ((uint64_t)K * cap < T) K = std::min(kMaxColours, (int)((T + cap - 1) / cap));
    cap = std::max(cap, (uint32_t)((T + K - 1) / K));
    std::vector<uint32_t> size(K, 0);
    for (uint32_t t : order) size[colour[t]]++;
    std::vector<std::array<uint64_t, 2>> vm(n_verts, {0ull, 0ull});
    auto mark = [&](uint32_t t, int c) {
        for (int k = 0; k < 4; ++k) {
            if (c < 64) vm[tets[4 * t + k]][0] |= 1ull << c;
            else vm[tets[4 * t + k]][1] |= 1ull << (c - 64);
        }
    };
    for (uint32_t t : order) mark(t, colour[t]);
    for (uint32_t t : order) {
        const int c = colour[t];
        if (size[c] <= cap) continue;
        uint64_t f0 = 0, f1 = 0;
        for (int k = 0; k < 4; ++k) {
            f0 |= vm[tets[4 * t + k]][0];
            f1 |= vm[tets[4 * t + k]][1];
        }
        int best = -1;
        for (int d = 0; d < K; ++d) {
            const bool used = d < 64 ? ((f0 >> d) & 1ull) : ((f1 >> (d - 64)) & 1ull);
            if (used || size[d] >= cap) continue;
            if (best < 0 || size[d] < size[best]) best = d;
        }
        if (best < 0) continue;
        // bit c stays set at t's vertices: conservative, as c is oversized
        // and takes no tets
        colour[t] = best;
        size[c]--;
        size[best]++;
        mark(t, best);
    }
    return K;
}

// Colours tets (given in `order`, a Morton order) so that no two tets of a
// colour share a vertex.  First-fit greedy, then a second pass with a size
// cap of ~T/K per colour to balance colour sizes.  Returns the colour count
// or -1 if more than kMaxColours are needed.
static int colour_tets(const std::vector<uint32_t>& tets, uint32_t n_verts, const std::vector<uint32_t>& order,
                       std::vector<int32_t>& colour, uint32_t size_cap = 0) {
    const size_t T = order.size();
    colour.assign(tets.size() / 4, -1);
    std::vector<std::array<uint64_t, 2>> vm(n_verts, {0ull, 0ull});
    auto pick = [&](uint32_t t, const std::vector<uint32_t>* size, uint32_t cap) -> int {
        uint64_t f0 = 0, f1 = 0;
        for (int k = 0; k < 4; ++k) {
            f0 |= vm[tets[4 * t + k]][0];
            f1 |= vm[tets[4 * t + k]][1];
        }
        int first_free = -1;
        for (int c = 0; c < kMaxColours; ++c) {
            bool used = c < 64 ? ((f0 >> c) & 1ull) : ((f1 >> (c - 64)) & 1ull);
            if (used) continue;
            if (first_free < 0) first_free = c;
            if (!size || (*size)[c] < cap) return c;
        }
        return first_free;
    };
    auto mark = [&](uint32_t t, int c) {
        for (int k = 0; k < 4; ++k) {
            if (c < 64) vm[tets[4 * t + k]][0] |= 1ull << c;
            else vm[tets[4 * t + k]][1] |= 1ull << (c - 64);
        }
    };
    auto greedy = [&](const std::vector<uint32_t>& ord, std::vector<int32_t>& col) -> int {
        for (auto& m : vm) m = {0ull, 0ull};
        int k = 0;
        for (uint32_t t : ord) {
            const int c = pick(t, nullptr, 0);
            if (c < 0) return -1;
            col[t] = c;
            mark(t, c);
            k = std::max(k, c + 1);
        }
        return k;
    };
    int K = greedy(order, colour);
    if (K < 0) return -1;
    // DSATUR (Brelaz 1979): colour next the uncoloured tet whose neighbours
    // (tets sharing a vertex) already use the most distinct colours, with
    // the smallest colour free at its vertices; kept when it needs fewer
    // colours than first-fit.  Saturations come from the vertex colour masks.
    if (T <= 4000000) {
        const uint32_t NV = n_verts;
        std::vector<uint32_t> inc_start(NV + 1, 0), inc;
        for (uint32_t t : order)
            for (int k = 0; k < 4; ++k) inc_start[tets[4 * t + k] + 1]++;
        for (uint32_t v = 0; v < NV; ++v) inc_start[v + 1] += inc_start[v];
        inc.resize(inc_start[NV]);
        {
            std::vector<uint32_t> fill(inc_start.begin(), inc_start.end() - 1);
            for (uint32_t t : order)
                for (int k = 0; k < 4; ++k) inc[fill[tets[4 * t + k]]++] = t;
        }
        for (auto& m : vm) m = {0ull, 0ull};
        std::vector<int32_t> cd(colour.size(), -1);
        std::vector<uint8_t> sat(colour.size(), 0);
        std::vector<std::vector<uint32_t>> bucket(kMaxColours + 1);
        auto saturation = [&](uint32_t t) {
            uint64_t f0 = 0, f1 = 0;
            for (int k = 0; k < 4; ++k) {
                f0 |= vm[tets[4 * t + k]][0];
                f1 |= vm[tets[4 * t + k]][1];
            }
            return (uint8_t)(__builtin_popcountll(f0) + __builtin_popcountll(f1));
        };
        // seed in reverse Morton order so the LIFO bucket starts at the first tet
        for (size_t i = order.size(); i-- > 0;) bucket[0].push_back(order[i]);
        int top = 0, Kd = 0;
        bool ok = true;
        for (size_t done = 0; done < T && ok;) {
            while (top > 0 && bucket[top].empty()) --top;
            if (bucket[top].empty()) break;
            const uint32_t t = bucket[top].back();
            bucket[top].pop_back();
            if (cd[t] >= 0 || sat[t] != top) continue;   // stale entry
            const int c = pick(t, nullptr, 0);
            if (c < 0) { ok = false; break; }
            cd[t] = c;
            mark(t, c);
            Kd = std::max(Kd, c + 1);
            ++done;
            for (int k = 0; k < 4; ++k) {
                const uint32_t v = tets[4 * t + k];
                for (uint32_t j = inc_start[v]; j < inc_start[v + 1]; ++j) {
                    const uint32_t u = inc[j];
                    if (cd[u] >= 0) continue;
                    const uint8_t su = saturation(u);
                    if (su != sat[u]) {
                        sat[u] = su;
                        bucket[su].push_back(u);
                        top = std::max(top, (int)su);
                    }
                }
            }
        }
        if (ok && Kd > 0 && Kd < K) {
            bool all = true;
            for (uint32_t t : order) all &= cd[t] >= 0;
            if (all) {
                colour.swap(cd);
                K = Kd;
            }
        }
    }
    // iterated greedy (Culberson): first-fit again over the tets listed class
    // by class never needs more colours and often needs fewer; the class
    // order varies between passes (reverse, largest first, smallest first)
    {
        const int passes = T <= 500000 ? 24 : T <= 4000000 ? 8 : 0;
        std::vector<int32_t> c2(colour.size(), -1);
        std::vector<uint32_t> ord(T);
        for (int pass = 0; pass < passes && K > 1; ++pass) {
            std::vector<uint32_t> size(K, 0);
            for (uint32_t t : order) size[colour[t]]++;
            std::vector<int> rank(K);
            for (int c = 0; c < K; ++c) rank[c] = c;
            if (pass % 3 == 0) std::reverse(rank.begin(), rank.end());
            else if (pass % 3 == 1) std::stable_sort(rank.begin(), rank.end(), [&](int a, int b) { return size[a] > size[b]; });
            else std::stable_sort(rank.begin(), rank.end(), [&](int a, int b) { return size[a] < size[b]; });
            std::vector<uint32_t> start(K + 1, 0);
            std::vector<int> pos(K);
            for (int r = 0; r < K; ++r) pos[rank[r]] = r;
            for (int c = 0; c < K; ++c) start[pos[c] + 1] = size[c];
            for (int r = 0; r < K; ++r) start[r + 1] += start[r];
            for (uint32_t t : order) ord[start[pos[colour[t]]]++] = t;   // Morton order kept inside a class
            const int K2 = greedy(ord, c2);
            if (K2 < 0 || K2 > K) break;
            colour.swap(c2);
            K = K2;
        }
    }
    // balance the classes: at most ~T/K (2% slack), or the size cap
    uint32_t cap = (uint32_t)std::ceil((double)T / K * 1.02) + 1;
    if (size_cap > 0) cap = std::min(cap, size_cap);
    K = balance_classes(tets, n_verts, order, colour, K, cap);
    return K;
}

// Gauss-Seidel sweep order of a scene: tets sorted by Morton code of their
// rest centroid, coloured, then ordered by (colour by decreasing size, model,
// Morton code).  `model` may be null (all StVK).  Outputs: order[k] = tet id
// projected k-th, offsets (K+1 colour starts), split[c] = first SNH slot of
// colour c.  Returns the colour count K or -1.
// A caller's colouring (hint[t] for every tet, e.g. the lattice colouring of
// a structured grid, which reaches the lower bound of tets meeting at a
// vertex where the greedy heuristics do not): -1 if some tet has none; -2 if
// two tets of one colour share a vertex or a colour is >= kMaxColours;
// otherwise the colour count, with the colours compacted to 0..K-1.
static int hint_colouring(const uint32_t* tets, uint32_t T, uint32_t V, const int32_t* hint,
                          std::vector<int32_t>& colour) {
    if (!hint) return -1;
    int32_t mx = -1;
    for (uint32_t t = 0; t < T; ++t) {
        if (hint[t] < 0) return -1;
        if (hint[t] >= kMaxColours) return -2;
        mx = std::max(mx, hint[t]);
    }
    std::vector<int32_t> remap(mx + 1, -1);
    int K = 0;
    for (uint32_t t = 0; t < T; ++t)
        if (remap[hint[t]] < 0) remap[hint[t]] = K++;
    colour.assign(T, 0);
    std::vector<std::array<uint64_t, 2>> vm(V, {0ull, 0ull});
    for (uint32_t t = 0; t < T; ++t) {
        const int c = remap[hint[t]];
        const uint64_t bit = 1ull << (c & 63);
        for (int k = 0; k < 4; ++k) {
            uint64_t& w = vm[tets[4ull * t + k]][c >> 6];
            if (w & bit) return -2;
            w |= bit;
        }
        colour[t] = c;
    }
    return K;
}

static int plan_sweep(const double* x0, uint32_t V, const uint32_t* tets, uint32_t T, const int32_t* model,
                      std::vector<uint32_t>& order, std::vector<uint32_t>& offsets, std::vector<uint32_t>& split,
                      const int32_t* hint = nullptr, bool* bad_hint = nullptr, uint32_t size_cap = 0) {
    auto mdl = [&](uint32_t t) { return model ? model[t] : (int32_t)SBS_MODEL_STVK; };
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (uint32_t i = 0; i < V; ++i)
        for (int k = 0; k < 3; ++k) {
            lo[k] = std::min(lo[k], x0[3ull * i + k]);
            hi[k] = std::max(hi[k], x0[3ull * i + k]);
        }
    std::vector<uint32_t> tm(T);
    for (uint32_t t = 0; t < T; ++t) {
        double c[3] = {0, 0, 0};
        for (int k = 0; k < 4; ++k)
            for (int a = 0; a < 3; ++a) c[a] += 0.25 * x0[3ull * tets[4ull * t + k] + a];
        tm[t] = morton(c, lo, hi);
    }
    std::vector<uint32_t> morder(T);
    std::iota(morder.begin(), morder.end(), 0u);
    std::stable_sort(morder.begin(), morder.end(), [&](uint32_t a, uint32_t b) { return tm[a] < tm[b]; });
    std::vector<uint32_t> tv(tets, tets + 4ull * T);
    std::vector<int32_t> colour, hinted;
    int K = colour_tets(tv, V, morder, colour, size_cap);
    const int Kh = hint_colouring(tets, T, V, hint, hinted);
    if (bad_hint) *bad_hint = Kh == -2;
    if (Kh > 0 && (K < 0 || Kh <= K)) {
        // the caller's colouring needs no more colours than the heuristics;
        // under a size cap its oversized classes are rebalanced as above
        K = Kh;
        colour.swap(hinted);
        if (size_cap > 0) {
            std::vector<uint32_t> csz(K, 0);
            for (uint32_t t = 0; t < T; ++t) csz[colour[t]]++;
            if (*std::max_element(csz.begin(), csz.end()) > size_cap)
                K = balance_classes(tv, V, morder, colour, K, size_cap);
        }
    }
    if (K < 0) return -1;
    std::vector<uint32_t> csize(K, 0);
    for (uint32_t t = 0; t < T; ++t) csize[colour[t]]++;
    std::vector<int> crank(K);
    std::iota(crank.begin(), crank.end(), 0);
    std::stable_sort(crank.begin(), crank.end(), [&](int a, int b) { return csize[a] > csize[b]; });
    std::vector<int> relabel(K);
    for (int r = 0; r < K; ++r) relabel[crank[r]] = r;
    std::vector<uint32_t> pos_in_m(T);
    for (uint32_t k = 0; k < T; ++k) pos_in_m[morder[k]] = k;
    order.resize(T);
    std::iota(order.begin(), order.end(), 0u);
    std::sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        int ca = relabel[colour[a]], cb = relabel[colour[b]];
        if (ca != cb) return ca < cb;
        if (mdl(a) != mdl(b)) return mdl(a) < mdl(b);
        return pos_in_m[a] < pos_in_m[b];
    });
    offsets.assign(K + 1, 0);
    split.assign(K, 0);
    uint32_t k = 0;
    for (int c = 0; c < K; ++c) {
        offsets[c] = k;
        while (k < T && relabel[colour[order[k]]] == c && mdl(order[k]) == SBS_MODEL_STVK) ++k;
        split[c] = k;
        while (k < T && relabel[colour[order[k]]] == c) ++k;
    }
    offsets[K] = k;
    return K;
}

extern "C" {

sbs_status sbs_gpu_plan_sweep(const double* x0, uint32_t n_verts, const uint32_t* tets, uint32_t n_tets,
                              const int32_t* models, const int32_t* colours, uint32_t* order, uint32_t* offsets,
                              uint32_t cap_offsets, uint32_t* n_colours) {
    if (!x0 || !tets || n_verts == 0 || n_tets == 0) return fail(nullptr, SBS_EINVAL, "plan: null/empty");
    for (uint64_t i = 0; i < 4ull * n_tets; ++i)
        if (tets[i] >= n_verts) return fail(nullptr, SBS_EINVAL, "plan: vertex index out of range");
    std::vector<uint32_t> ord, off, split;
    bool bad = false;
    const int K = plan_sweep(x0, n_verts, tets, n_tets, models, ord, off, split, colours, &bad);
    if (bad) return fail(nullptr, SBS_EINVAL, "plan: two tets of one given colour share a vertex");
    if (K < 0) return fail(nullptr, SBS_ECOLOUR, "constraint graph needs more than 128 colours");
    if (n_colours) *n_colours = (uint32_t)K;
    if (order) std::copy(ord.begin(), ord.end(), order);
    if (offsets) {
        if (cap_offsets < (uint32_t)K + 1) return fail(nullptr, SBS_EINVAL, "plan: offsets capacity");
        std::copy(off.begin(), off.end(), offsets);
    }
    return SBS_OK;
}

const char* sbs_gpu_status_string(sbs_status s) {
    switch (s) {
        case SBS_OK: return "ok";
        case SBS_EINVAL: return "invalid argument";
        case SBS_ECUDA: return "CUDA error";
        case SBS_ETIMEOUT: return "device wait timed out";
        case SBS_ENAN: return "non-finite state";
        case SBS_ESTATE: return "call not valid in this state";
        case SBS_ENOMEM: return "out of device memory";
        case SBS_ECOLOUR: return "too many colours";
    }
    return "unknown";
}

const char* sbs_gpu_last_error(const sbs_gpu* h) { return h ? h->last_error.c_str() : g_err.c_str(); }

sbs_status sbs_gpu_params_default(sbs_gpu_params* p) {
    if (!p) return SBS_EINVAL;
    std::memset(p, 0, sizeof(*p));
    p->compliance = 1e-4;
    p->damping = 0.0;
    p->collision_compliance = 1e-8;
    p->gravity[0] = 0.0;
    p->gravity[1] = -9.81;
    p->gravity[2] = 0.0;
    p->gravity_mode = SBS_GRAVITY_ACCELERATION;
    p->device = 0;
    p->exec_mode = SBS_EXEC_AUTO;
    p->block_size = 0;
    p->ctas_per_sm = 0;
    p->tail_threshold = -1;
    p->body_contacts = 0;
    p->hash_cell = 0.0f;
    p->candidate_capacity = 0;
    p->check_finite = 1;
    p->stage_records = 1;
    p->wait_limit_us = 0;
    p->colour_size_cap = 0;
    return SBS_OK;
}

sbs_status sbs_gpu_create(const sbs_gpu_params* p, sbs_gpu** out) {
    if (!out) return SBS_EINVAL;
    *out = nullptr;
    sbs_gpu_params prm;
    if (p) prm = *p;
    else sbs_gpu_params_default(&prm);
    if (prm.gravity_mode != 0 && prm.gravity_mode != 1) return fail(nullptr, SBS_EINVAL, "gravity_mode");
    if (prm.exec_mode < 0 || prm.exec_mode > 4) return fail(nullptr, SBS_EINVAL, "exec_mode");
    if (prm.wait_limit_us < 0) return fail(nullptr, SBS_EINVAL, "wait_limit_us");
    if (prm.colour_size_cap < -1) return fail(nullptr, SBS_EINVAL, "colour_size_cap");
    if (prm.stage_records < 0 || prm.stage_records > 2) return fail(nullptr, SBS_EINVAL, "stage_records");
    if (prm.block_size != 0 && (prm.block_size < 32 || prm.block_size > 512 || prm.block_size % 32))
        return fail(nullptr, SBS_EINVAL, "block_size must be a multiple of 32 in [32, 512]");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(nullptr, SBS_ECUDA, "no CUDA device available");
    if (prm.device < 0 || prm.device >= ndev) return fail(nullptr, SBS_EINVAL, "device ordinal out of range");
    sbs_gpu* h = new sbs_gpu();
    h->prm = prm;
    cudaError_t e = cudaSetDevice(prm.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->n_sm, cudaDevAttrMultiProcessorCount, prm.device);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
    if (e != cudaSuccess) {
        std::string m = cudaGetErrorString(e);
        sbs_gpu_destroy(h);
        return fail(nullptr, SBS_ECUDA, "create: " + m);
    }
    *out = h;
    return SBS_OK;
}

sbs_status sbs_gpu_add_body(sbs_gpu* h, const double* x0, const double* x_init, uint32_t n_verts,
                            const uint32_t* tets, uint32_t n_tets, const sbs_gpu_material* mat,
                            const double* mass, int32_t* body_id) {
    if (!h || !x0 || !tets || !mat || n_verts == 0 || n_tets == 0) return fail(h, SBS_EINVAL, "add_body: null/empty");
    if (h->finalized) return fail(h, SBS_ESTATE, "add_body after finalize");
    if (mat->model != SBS_MODEL_STVK && mat->model != SBS_MODEL_SNH) return fail(h, SBS_EINVAL, "material model");
    if (!(mat->young > 0) || !(mat->poisson > -1.0 && mat->poisson < 0.5) || !(mat->density >= 0))
        return fail(h, SBS_EINVAL, "material parameters");
    for (uint64_t i = 0; i < 4ull * n_tets; ++i)
        if (tets[i] >= n_verts) return fail(h, SBS_EINVAL, "tet vertex index out of range");
    for (uint64_t i = 0; i < 3ull * n_verts; ++i)
        if (!std::isfinite(x0[i]) || (x_init && !std::isfinite(x_init[i])))
            return fail(h, SBS_EINVAL, "non-finite position");
    BodyHost b;
    b.v0 = (uint32_t)(h->x0.size() / 3);
    b.nv = n_verts;
    b.t0 = (uint32_t)(h->tets.size() / 4);
    b.nt = n_tets;
    if ((uint64_t)b.v0 + n_verts >= (1ull << 31) || (uint64_t)b.t0 + n_tets >= (1ull << 31))
        return fail(h, SBS_EINVAL, "scene too large");
    h->x0.insert(h->x0.end(), x0, x0 + 3ull * n_verts);
    if (x_init) h->xinit.insert(h->xinit.end(), x_init, x_init + 3ull * n_verts);
    else h->xinit.insert(h->xinit.end(), x0, x0 + 3ull * n_verts);
    h->vinit.resize(h->xinit.size(), 0.0f);
    // lumped masses: density * |V0| / 4 per incident tet
    std::vector<double> m(n_verts, 0.0);
    for (uint32_t t = 0; t < n_tets; ++t) {
        const uint32_t* q = tets + 4ull * t;
        double D[3][3];
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) D[r][c] = x0[3ull * q[c] + r] - x0[3ull * q[3] + r];
        double det = D[0][0] * (D[1][1] * D[2][2] - D[1][2] * D[2][1]) - D[0][1] * (D[1][0] * D[2][2] - D[1][2] * D[2][0]) +
                     D[0][2] * (D[1][0] * D[2][1] - D[1][1] * D[2][0]);
        if (!(std::fabs(det) > 0)) return fail(h, SBS_EINVAL, "degenerate rest tet");
        double V = std::fabs(det / 6.0);
        for (int k = 0; k < 4; ++k) m[q[k]] += mat->density * V / 4.0;
    }
    for (uint32_t i = 0; i < n_verts; ++i) {
        h->mass.push_back(mass ? mass[i] : m[i]);
        h->user_mass.push_back(mass ? 1 : 0);
        h->kin_group.push_back(-1);
    }
    const double mu = mat->young / (2.0 * (1.0 + mat->poisson));
    const double lam = mat->young * mat->poisson / ((1.0 + mat->poisson) * (1.0 - 2.0 * mat->poisson));
    for (uint64_t i = 0; i < 4ull * n_tets; ++i) h->tets.push_back(b.v0 + tets[i]);
    for (uint32_t t = 0; t < n_tets; ++t) {
        h->tet_model.push_back(mat->model);
        h->tet_hint.push_back(-1);
        h->tet_mu.push_back(mu);
        h->tet_lam.push_back(lam);
    }
    h->bodies.push_back(std::move(b));
    if (body_id) *body_id = (int32_t)h->bodies.size() - 1;
    return SBS_OK;
}

sbs_status sbs_gpu_set_tet_colours(sbs_gpu* h, int32_t body, const uint32_t* colours) {
    if (!h || !colours) return fail(h, SBS_EINVAL, "set_tet_colours: null");
    if (h->finalized) return fail(h, SBS_ESTATE, "set_tet_colours after finalize");
    if (body < 0 || body >= (int32_t)h->bodies.size()) return fail(h, SBS_EINVAL, "body id");
    const BodyHost& b = h->bodies[body];
    for (uint32_t t = 0; t < b.nt; ++t)
        if (colours[t] >= (uint32_t)kMaxColours) return fail(h, SBS_EINVAL, "set_tet_colours: colour >= 128");
    for (uint32_t t = 0; t < b.nt; ++t) h->tet_hint[b.t0 + t] = (int32_t)colours[t];
    return SBS_OK;
}

sbs_status sbs_gpu_pin_vertices(sbs_gpu* h, int32_t body, const uint32_t* verts, uint32_t n) {
    if (!h || (n && !verts)) return fail(h, SBS_EINVAL, "pin: null");
    if (h->finalized) return fail(h, SBS_ESTATE, "pin after finalize");
    if (body < 0 || body >= (int32_t)h->bodies.size()) return fail(h, SBS_EINVAL, "pin: body id");
    const BodyHost& b = h->bodies[body];
    for (uint32_t i = 0; i < n; ++i) {
        if (verts[i] >= b.nv) return fail(h, SBS_EINVAL, "pin: vertex id");
        h->mass[b.v0 + verts[i]] = 0.0;
    }
    return SBS_OK;
}

sbs_status sbs_gpu_add_kinematic_rotation(sbs_gpu* h, int32_t body, const uint32_t* verts, uint32_t n,
                                          const double center[3], const double axis[3], double omega) {
    if (!h || (n && !verts) || !center || !axis) return fail(h, SBS_EINVAL, "kinematic: null");
    if (h->finalized) return fail(h, SBS_ESTATE, "kinematic after finalize");
    if (body < 0 || body >= (int32_t)h->bodies.size()) return fail(h, SBS_EINVAL, "kinematic: body id");
    if (h->groups.size() >= (size_t)kMaxKinGroups) return fail(h, SBS_EINVAL, "too many kinematic groups");
    double l = std::sqrt(axis[0] * axis[0] + axis[1] * axis[1] + axis[2] * axis[2]);
    if (!(l > 0)) return fail(h, SBS_EINVAL, "kinematic: zero axis");
    KinGroup g;
    g.cx = (float)center[0]; g.cy = (float)center[1]; g.cz = (float)center[2];
    g.ax = (float)(axis[0] / l); g.ay = (float)(axis[1] / l); g.az = (float)(axis[2] / l);
    g.omega = omega;
    const BodyHost& b = h->bodies[body];
    for (uint32_t i = 0; i < n; ++i)
        if (verts[i] >= b.nv) return fail(h, SBS_EINVAL, "kinematic: vertex id");
    h->groups.push_back(g);
    for (uint32_t i = 0; i < n; ++i) {
        h->kin_group[b.v0 + verts[i]] = (int32_t)h->groups.size() - 1;
        h->mass[b.v0 + verts[i]] = 0.0;
    }
    return SBS_OK;
}

sbs_status sbs_gpu_set_external_acceleration(sbs_gpu* h, int32_t body, const float* a) {
    if (!h || !a) return fail(h, SBS_EINVAL, "acc: null");
    if (h->finalized) return fail(h, SBS_ESTATE, "acc after finalize");
    if (body < 0 || body >= (int32_t)h->bodies.size()) return fail(h, SBS_EINVAL, "acc: body id");
    const BodyHost& b = h->bodies[body];
    h->acc.resize(h->x0.size(), 0.0f);
    std::copy(a, a + 3ull * b.nv, h->acc.begin() + 3ull * b.v0);
    h->has_acc = true;
    return SBS_OK;
}

sbs_status sbs_gpu_add_ground_plane(sbs_gpu* h, const double n[3], double d) {
    if (!h || !n) return fail(h, SBS_EINVAL, "plane: null");
    if (h->finalized) return fail(h, SBS_ESTATE, "plane after finalize");
    if (h->planes.size() + h->grids.size() >= (size_t)kMaxPlanes) return fail(h, SBS_EINVAL, "too many planes");
    if (!h->grids.empty()) return fail(h, SBS_ESTATE, "add planes before sdf grids");
    double l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
    if (!(l > 0) || !std::isfinite(d)) return fail(h, SBS_EINVAL, "plane normal");
    h->planes.push_back(Plane{(float)(n[0] / l), (float)(n[1] / l), (float)(n[2] / l), (float)(d / l)});
    return SBS_OK;
}

sbs_status sbs_gpu_add_distance_constraints(sbs_gpu* h, const uint32_t* ids, uint32_t n, double alpha,
                                            double beta) {
    if (!h || (n && !ids)) return fail(h, SBS_EINVAL, "distance: null");
    if (h->finalized) return fail(h, SBS_ESTATE, "distance constraints after finalize");
    if (!(alpha >= 0.0) || !(beta >= 0.0) || !std::isfinite(alpha) || !std::isfinite(beta))
        return fail(h, SBS_EINVAL, "distance: alpha and beta must be finite and >= 0");
    std::vector<uint32_t> v;
    std::vector<float4> q;
    for (uint32_t k = 0; k < n; ++k) {
        const uint32_t b1 = ids[4ull * k], b2 = ids[4ull * k + 1], v1 = ids[4ull * k + 2], v2 = ids[4ull * k + 3];
        if (b1 >= h->bodies.size() || b2 >= h->bodies.size() || v1 >= h->bodies[b1].nv || v2 >= h->bodies[b2].nv)
            return fail(h, SBS_EINVAL, "distance: body or vertex id out of range");
        const uint32_t g1 = h->bodies[b1].v0 + v1, g2 = h->bodies[b2].v0 + v2;
        if (g1 == g2) return fail(h, SBS_EINVAL, "distance: both ends are the same vertex");
        double l2 = 0.0;
        for (int c = 0; c < 3; ++c) {
            const double dd = h->x0[3ull * g1 + c] - h->x0[3ull * g2 + c];
            l2 += dd * dd;
        }
        v.push_back(g1);
        v.push_back(g2);
        q.push_back(make_float4((float)std::sqrt(l2), (float)alpha, (float)beta, 0.0f));
    }
    h->dist_v.insert(h->dist_v.end(), v.begin(), v.end());
    h->dist_p.insert(h->dist_p.end(), q.begin(), q.end());
    return SBS_OK;
}

// First-fit edge colouring in input order: an edge takes the smallest colour
// neither end has used; colours are then listed largest first, input order
// kept inside a colour.  Returns the colour count, or -1 above kMaxEdgeColours.
static int colour_edges(const std::vector<uint32_t>& ends, uint32_t V, std::vector<uint32_t>& order,
                        std::vector<uint32_t>& offsets) {
    const size_t E = ends.size() / 2;
    std::vector<uint64_t> used(V, 0);
    std::vector<int> col(E);
    int K = 0;
    for (size_t k = 0; k < E; ++k) {
        const uint64_t busy = used[ends[2 * k]] | used[ends[2 * k + 1]];
        if (busy == ~0ull) return -1;
        int c = 0;
        while (busy >> c & 1ull) ++c;
        col[k] = c;
        used[ends[2 * k]] |= 1ull << c;
        used[ends[2 * k + 1]] |= 1ull << c;
        K = std::max(K, c + 1);
    }
    std::vector<uint32_t> size(K, 0);
    for (int c : col) size[c]++;
    std::vector<int> rank(K);
    for (int c = 0; c < K; ++c) rank[c] = c;
    std::stable_sort(rank.begin(), rank.end(), [&](int a, int b) { return size[a] > size[b]; });
    std::vector<int> pos(K);
    for (int r = 0; r < K; ++r) pos[rank[r]] = r;
    offsets.assign(K + 1, 0);
    for (int c = 0; c < K; ++c) offsets[pos[c] + 1] = size[c];
    for (int r = 0; r < K; ++r) offsets[r + 1] += offsets[r];
    order.assign(E, 0);
    std::vector<uint32_t> fill(offsets.begin(), offsets.end() - 1);
    for (size_t k = 0; k < E; ++k) order[fill[pos[col[k]]]++] = (uint32_t)k;
    return K;
}

sbs_status sbs_gpu_set_body_velocity(sbs_gpu* h, int32_t body, const double v[3]) {
    if (!h || !v) return fail(h, SBS_EINVAL, "velocity: null");
    if (h->finalized) return fail(h, SBS_ESTATE, "initial velocity after finalize (use sbs_gpu_set_state)");
    if (body < 0 || body >= (int32_t)h->bodies.size()) return fail(h, SBS_EINVAL, "body id");
    if (!std::isfinite(v[0]) || !std::isfinite(v[1]) || !std::isfinite(v[2])) return fail(h, SBS_EINVAL, "velocity");
    const BodyHost& b = h->bodies[body];
    for (uint32_t i = 0; i < b.nv; ++i)
        for (int k = 0; k < 3; ++k) h->vinit[3ull * (b.v0 + i) + k] = (float)v[k];
    return SBS_OK;
}

static sbs_status add_grid(sbs_gpu* h, const float* values, const uint32_t nodes[3], const double origin[3],
                           const double spacing[3], int cubic) {
    if (!h || !values || !nodes || !origin || !spacing) return fail(h, SBS_EINVAL, "sdf grid: null");
    if (h->finalized) return fail(h, SBS_ESTATE, "sdf grid after finalize");
    if (h->grids.size() >= (size_t)kMaxGrids) return fail(h, SBS_EINVAL, "too many sdf grids");
    if (h->planes.size() + h->grids.size() >= (size_t)kMaxPlanes)
        return fail(h, SBS_EINVAL, "too many environment bodies (planes + grids)");
    sbs_gpu::GridHost g;
    for (int k = 0; k < 3; ++k) {
        if (nodes[k] < 2 || nodes[k] > 4096) return fail(h, SBS_EINVAL, "sdf grid: 1..4095 cells per axis");
        if (!(spacing[k] > 0) || !std::isfinite(origin[k])) return fail(h, SBS_EINVAL, "sdf grid: spacing/origin");
        g.n[k] = nodes[k];
        g.o[k] = origin[k];
        g.h[k] = spacing[k];
    }
    const size_t n = cubic ? sdf_cubic_count(nodes[0], nodes[1], nodes[2]) : (size_t)nodes[0] * nodes[1] * nodes[2];
    g.v.assign(values, values + n);
    g.cubic = cubic;
    for (float f : g.v)
        if (!std::isfinite(f)) return fail(h, SBS_EINVAL, "sdf grid: non-finite value");
    h->grids.push_back(std::move(g));
    return SBS_OK;
}

sbs_status sbs_gpu_add_sdf_grid(sbs_gpu* h, const float* values, const uint32_t nodes[3], const double origin[3],
                                const double spacing[3]) {
    return add_grid(h, values, nodes, origin, spacing, 0);
}

sbs_status sbs_gpu_add_sdf_grid_cubic(sbs_gpu* h, const float* values, const uint32_t cells[3], const double origin[3],
                                      const double spacing[3]) {
    if (!cells) return fail(h, SBS_EINVAL, "sdf grid: null");
    for (int k = 0; k < 3; ++k)
        if (cells[k] == 0 || cells[k] > 4095) return fail(h, SBS_EINVAL, "sdf grid: 1..4095 cells per axis");
    const uint32_t nodes[3] = {cells[0] + 1, cells[1] + 1, cells[2] + 1};
    return add_grid(h, values, nodes, origin, spacing, 1);
}

extern "C" sbs_status sbs_gpu_sdf_cubic_from_mesh(const double* verts, uint32_t n_verts, const uint32_t* tris,
                                                  uint32_t n_tris, const double lo[3], const double hi[3],
                                                  const uint32_t cells[3], float* values);

sbs_status sbs_gpu_add_environment_mesh(sbs_gpu* h, const double* verts, uint32_t n_verts, const uint32_t* tris,
                                        uint32_t n_tris, const double domain_lo[3], const double domain_hi[3],
                                        const uint32_t cells[3]) {
    if (!h || !verts || !tris || !domain_lo || !domain_hi || !cells) return fail(h, SBS_EINVAL, "environment: null");
    // the domain as environment_body_t extends it (environment_body.cpp:53-63):
    // for every mesh vertex, grow the box over all vertices and pad both
    // corners by 1e-3 of the current diagonal
    double lo[3] = {domain_lo[0], domain_lo[1], domain_lo[2]}, hi[3] = {domain_hi[0], domain_hi[1], domain_hi[2]};
    for (uint32_t a = 0; a < n_verts; ++a) {
        for (uint32_t b = 0; b < n_verts; ++b)
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], verts[3ull * b + k]);
                hi[k] = std::max(hi[k], verts[3ull * b + k]);
            }
        const double dg = std::sqrt((hi[0] - lo[0]) * (hi[0] - lo[0]) + (hi[1] - lo[1]) * (hi[1] - lo[1]) +
                                    (hi[2] - lo[2]) * (hi[2] - lo[2]));
        for (int k = 0; k < 3; ++k) {
            hi[k] += 1e-3 * dg;
            lo[k] -= 1e-3 * dg;
        }
    }
    for (int k = 0; k < 3; ++k)
        if (cells[k] == 0 || cells[k] > 4095) return fail(h, SBS_EINVAL, "environment: 1..4095 cells per axis");
    // the cubic Lagrange grid of environment_body.cpp:72-73
    std::vector<float> v(sdf_cubic_count(cells[0] + 1, cells[1] + 1, cells[2] + 1));
    const sbs_status s = sbs_gpu_sdf_cubic_from_mesh(verts, n_verts, tris, n_tris, lo, hi, cells, v.data());
    if (s) return fail(h, s, "environment: bad mesh or domain");
    const double sp[3] = {(hi[0] - lo[0]) / cells[0], (hi[1] - lo[1]) / cells[1], (hi[2] - lo[2]) / cells[2]};
    return sbs_gpu_add_sdf_grid_cubic(h, v.data(), cells, lo, sp);
}

static sbs_status upload(sbs_gpu* h, void* dst, const void* src, size_t bytes) {
    if (bytes == 0) return SBS_OK;
    CU(h, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->st));
    return SBS_OK;
}

static void fill_params(sbs_gpu* h, StepParams& p, double dt, uint32_t substeps, uint32_t iterations) {
    p = h->base;
    p.dt_d = dt;
    p.dt = (float)dt;
    p.inv_dt = (float)(1.0 / dt);
    p.inv_dt2 = (float)(1.0 / (dt * dt));
    p.stvk_alpha_tilde = (float)(h->prm.compliance / (dt * dt));
    const double at = h->prm.compliance / (dt * dt), bt = h->prm.damping * dt * dt;
    p.stvk_gamma = (float)(at * bt / dt);
    p.stvk_damping = h->prm.damping != 0.0 ? 1 : 0;
    p.contact_alpha_tilde = (float)(h->prm.collision_compliance / (dt * dt));
    p.substeps = (int)substeps;
    p.iterations = (int)iterations;
}

// Wavefront mode.  The vertex slots (per-body Morton order) are cut into G
// equal ranges, one per CTA; a tet belongs to the CTA of its lowest vertex
// slot, so a CTA covers the same region of the mesh in every colour.  Outputs
// per (colour c, CTA b) the tet slots b projects in c (CSR: start[c * (G+1) + b]
// into idx) and, per CTA, the CTAs whose tets share a vertex with its own.
static void wave_partition(const std::vector<uint4>& tid, const std::vector<uint32_t>& offsets, int K, int G,
                           uint32_t V, std::vector<uint32_t>& wstart, std::vector<uint32_t>& widx,
                           std::vector<uint32_t>& nstart, std::vector<uint32_t>& nlist) {
    const size_t T = tid.size();
    std::vector<uint32_t> owner(T);
    for (size_t k = 0; k < T; ++k) {
        const uint4 q = tid[k];
        const uint32_t m = std::min(std::min(q.x, q.y), std::min(q.z, q.w));
        owner[k] = (uint32_t)((uint64_t)m * G / V);
    }
    wstart.assign((size_t)K * (G + 1), 0);
    widx.resize(T);
    for (int c = 0; c < K; ++c) {
        uint32_t* st = &wstart[(size_t)c * (G + 1)];
        for (uint32_t k = offsets[c]; k < offsets[c + 1]; ++k) st[owner[k] + 1]++;
        st[0] = offsets[c];
        for (int b = 0; b < G; ++b) st[b + 1] += st[b];
        std::vector<uint32_t> fill(st, st + G);
        for (uint32_t k = offsets[c]; k < offsets[c + 1]; ++k) widx[fill[owner[k]]++] = k;
    }
    std::vector<uint64_t> pairs;   // vertex * G + cta
    pairs.reserve(T * 4);
    for (size_t k = 0; k < T; ++k) {
        const uint4 q = tid[k];
        pairs.push_back((uint64_t)q.x * G + owner[k]);
        pairs.push_back((uint64_t)q.y * G + owner[k]);
        pairs.push_back((uint64_t)q.z * G + owner[k]);
        pairs.push_back((uint64_t)q.w * G + owner[k]);
    }
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    const size_t words = ((size_t)G + 63) / 64;
    std::vector<uint64_t> bits((size_t)G * words, 0);
    std::vector<uint32_t> ctas;
    for (size_t i = 0; i < pairs.size();) {
        const uint64_t v = pairs[i] / G;
        ctas.clear();
        while (i < pairs.size() && pairs[i] / G == v) ctas.push_back((uint32_t)(pairs[i++] % G));
        for (uint32_t a : ctas)
            for (uint32_t b : ctas)
                if (a != b) bits[(size_t)a * words + b / 64] |= 1ull << (b % 64);
    }
    nstart.assign(G + 1, 0);
    nlist.clear();
    for (int a = 0; a < G; ++a) {
        for (int b = 0; b < G; ++b)
            if (bits[(size_t)a * words + b / 64] >> (b % 64) & 1ull) nlist.push_back((uint32_t)b);
        nstart[a + 1] = (uint32_t)nlist.size();
    }
}

sbs_status sbs_gpu_finalize(sbs_gpu* h) {
    if (!h) return SBS_EINVAL;
    if (h->finalized) return fail(h, SBS_ESTATE, "finalize twice");
    if (h->bodies.empty()) return fail(h, SBS_ESTATE, "finalize without bodies");
    CU(h, cudaSetDevice(h->prm.device));
    const uint32_t V = (uint32_t)(h->x0.size() / 3), T = (uint32_t)(h->tets.size() / 4);
    h->n_verts = V;
    h->n_tets = T;
    // 1. per-body Morton order of vertices (bodies stay contiguous)
    std::vector<uint32_t> old_to_new(V), new_to_old(V);
    for (BodyHost& b : h->bodies) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (uint32_t i = 0; i < b.nv; ++i)
            for (int k = 0; k < 3; ++k) {
                lo[k] = std::min(lo[k], h->x0[3ull * (b.v0 + i) + k]);
                hi[k] = std::max(hi[k], h->x0[3ull * (b.v0 + i) + k]);
            }
        std::vector<std::pair<uint32_t, uint32_t>> key(b.nv);
        for (uint32_t i = 0; i < b.nv; ++i) key[i] = {morton(&h->x0[3ull * (b.v0 + i)], lo, hi), i};
        std::stable_sort(key.begin(), key.end());
        b.new_to_old.resize(b.nv);
        b.old_to_new.resize(b.nv);
        for (uint32_t n = 0; n < b.nv; ++n) {
            b.new_to_old[n] = key[n].second;
            b.old_to_new[key[n].second] = n;
            old_to_new[b.v0 + key[n].second] = b.v0 + n;
            new_to_old[b.v0 + n] = b.v0 + key[n].second;
        }
    }
    h->all_bodies.v0 = 0;
    h->all_bodies.nv = V;
    h->all_bodies.t0 = 0;
    h->all_bodies.nt = T;
    h->all_bodies.old_to_new = old_to_new;
    h->all_bodies.new_to_old = new_to_old;
    // 2. groups of consecutive bodies for the cluster-resident mode: every
    //    group must fit the shared memory of one cluster (<= 16 CTAs)
    const int P = (int)h->planes.size();
    int smem_optin = 0;
    CU(h, cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->prm.device));
    // per vertex: its state and contact records, plus the multipliers of the
    // tets it brings (T/V + 1 tets per vertex, 8 bytes each)
    const size_t per_v = cluster_smem_bytes(1, P, h->prm.body_contacts ? 1 : 0, 0) +
                         8 * ((size_t)T / std::max<uint32_t>(V, 1) + 1);
    uint32_t cap_slice = (uint32_t)((size_t)(smem_optin - 4096) / per_v);
    int shrink_tries = 0;
    uint32_t max_body = 0;
    for (const BodyHost& b : h->bodies) max_body = std::max(max_body, b.nv);
    // a plan whose cluster turns out not to be launchable is redone: with
    // smaller vertex slices when the final multiplier slices overflow the
    // shared memory, else (or after a few tries) with the cluster mode excluded
    // distance constraints may join any two bodies: they run in the global modes only
    bool allow_cluster = h->prm.exec_mode != SBS_EXEC_GRAPH && h->prm.exec_mode != SBS_EXEC_PERSISTENT &&
                         h->prm.exec_mode != SBS_EXEC_WAVEFRONT && h->dist_p.empty() && h->grids.empty();
    if (!h->grids.empty() && h->prm.exec_mode == SBS_EXEC_CLUSTER)
        return fail(h, SBS_EINVAL, "sdf grids do not run in the cluster-resident mode");
    if (!h->dist_p.empty() && h->prm.exec_mode == SBS_EXEC_CLUSTER)
        return fail(h, SBS_EINVAL, "distance constraints do not run in the cluster-resident mode");
plan_again:
    h->seg_split.clear();
    h->cl_size = 1;
    while (h->cl_size < 16 && (uint64_t)h->cl_size * cap_slice < max_body) h->cl_size *= 2;
    h->cl_feasible = (uint64_t)h->cl_size * cap_slice >= max_body && allow_cluster;
    h->cl_groups.clear();
    if (h->cl_feasible) {
        const uint64_t cap = (uint64_t)h->cl_size * cap_slice;
        uint32_t b0 = 0, nv = 0;
        for (uint32_t bi = 0; bi < h->bodies.size(); ++bi) {
            if (nv + h->bodies[bi].nv > cap && bi > b0) {
                h->cl_groups.push_back({b0, bi});
                b0 = bi;
                nv = 0;
            }
            nv += h->bodies[bi].nv;
        }
        h->cl_groups.push_back({b0, (uint32_t)h->bodies.size()});
        // groups that cannot all be resident at once run in rounds, each
        // paying the whole frame's chain of barriers; the global sweep is then
        // faster (measured on 512 boxes: 30 ms in rounds against 17 ms), so
        // several groups are planned only when they fit in one round
        if (h->cl_groups.size() > 1) {
            const size_t est = std::min<size_t>((size_t)smem_optin, (size_t)cap_slice * per_v + 4096);
            const int blk = h->prm.block_size ? std::min(h->prm.block_size, kClusterMaxBlock) : 256;
            int active = 0;
            if (cluster_configure(blk, est) != cudaSuccess ||
                cluster_max_active(h->cl_size, blk, est, &active) != cudaSuccess ||
                (size_t)active < h->cl_groups.size()) {
                cudaGetLastError();
                if (h->prm.exec_mode != SBS_EXEC_CLUSTER) {
                    h->cl_feasible = false;
                    h->cl_groups.clear();
                }
            }
        }
    }
    // 3. sweep order: per group (several groups) or over the whole scene:
    //    colour (size-descending), model, Morton code
    std::vector<uint32_t> split;
    std::vector<uint32_t> gcol_start, gcol_split;
    std::vector<GroupDesc> gdesc;
    int K = 0;
    if (h->cl_feasible && h->cl_groups.size() > 1) {
        h->tet_order.clear();
        h->colour_offsets.assign(1, 0);
        for (auto& gr : h->cl_groups) {
            const BodyHost& bf = h->bodies[gr.first];
            const BodyHost& bl = h->bodies[gr.second - 1];
            const uint32_t ov0 = bf.v0, onv = bl.v0 + bl.nv - bf.v0;
            const uint32_t t0 = bf.t0, nt = bl.t0 + bl.nt - bf.t0;
            std::vector<uint32_t> lt(4ull * nt);
            for (uint64_t i = 0; i < 4ull * nt; ++i) lt[i] = h->tets[4ull * t0 + i] - ov0;
            std::vector<uint32_t> ord, off, spl;
            bool bad = false;
            const int Kg = plan_sweep(&h->x0[3ull * ov0], onv, lt.data(), nt, &h->tet_model[t0], ord, off, spl,
                                      &h->tet_hint[t0], &bad);
            if (bad) return fail(h, SBS_EINVAL, "two tets of one given colour share a vertex");
            if (Kg < 0) return fail(h, SBS_ECOLOUR, "constraint graph needs more than 128 colours");
            const uint32_t base = (uint32_t)h->tet_order.size();
            GroupDesc g;
            g.v0 = ov0;  // library ids keep the add order of bodies
            g.nv = onv;
            g.col_base = (uint32_t)gcol_start.size();
            g.n_col = (uint32_t)Kg;
            gdesc.push_back(g);
            for (uint32_t k : ord) h->tet_order.push_back(t0 + k);
            for (int c = 0; c <= Kg; ++c) gcol_start.push_back(base + off[c]);
            for (int c = 0; c < Kg; ++c) gcol_split.push_back(base + spl[c]);
            for (int c = 0; c < Kg; ++c) h->seg_split.push_back(base + spl[c]);
            gcol_split.push_back(base + off[Kg]);
            for (int c = 1; c <= Kg; ++c) h->colour_offsets.push_back(base + off[c]);
            K = std::max(K, Kg);
        }
        h->global_modes = false;   // tets are group-major: only the cluster mode runs them
        h->n_colours = (uint32_t)(h->colour_offsets.size() - 1);
    } else {
        bool bad = false;
        // without the cluster mode, colours of at most one tet per resident
        // thread of the persistent kernel (512 per SM at its 128 registers)
        const uint32_t size_cap = h->cl_feasible || h->prm.colour_size_cap < 0 ? 0u
                                  : h->prm.colour_size_cap > 0           ? (uint32_t)h->prm.colour_size_cap
                                                                         : (uint32_t)h->n_sm * 512u;
        K = plan_sweep(h->x0.data(), V, h->tets.data(), T, h->tet_model.data(), h->tet_order, h->colour_offsets,
                       split, h->tet_hint.data(), &bad, size_cap);
        if (bad) return fail(h, SBS_EINVAL, "two tets of one given colour share a vertex");
        if (K < 0) return fail(h, SBS_ECOLOUR, "constraint graph needs more than 128 colours");
        h->n_colours = (uint32_t)K;
        h->global_modes = true;
        h->seg_split = split;
        if (h->cl_feasible) {
            GroupDesc g;
            g.v0 = 0;
            g.nv = V;
            g.col_base = 0;
            g.n_col = (uint32_t)K;
            gdesc.push_back(g);
            gcol_start = h->colour_offsets;
            gcol_split = split;
            gcol_split.push_back(T);
        }
    }
    // single group: enough CTAs that a colour is about one tet per thread
    if (h->cl_feasible && gdesc.size() == 1) {
        uint32_t maxc = 0;
        for (size_t c = 0; c + 1 < gcol_start.size(); ++c) maxc = std::max(maxc, gcol_start[c + 1] - gcol_start[c]);
        while (h->cl_size < 16 && (uint64_t)h->cl_size * 256 < maxc) h->cl_size *= 2;
    }
    // cluster mode: every tet goes to the CTA whose vertex slice holds most
    // of its vertices (gathers then mostly hit the CTA's own shared memory).
    // A colour phase lasts as long as its busiest CTA, so when that leaves a
    // CTA more tets than 256 threads (or an even split's share, ceil(colour
    // size / C), rounded up to warps) cover in one pass, the colour is split
    // evenly: its tets ordered by that
    // majority CTA and, inside it, from those with most vertices in the
    // previous CTA's slice to those with most in the next one, then cut into
    // C consecutive runs - the tets that change CTA are those at the edges of
    // a region, sharing vertices with the CTA they move to.  Within a colour
    // tets are reordered by owner, which leaves each colour's tet set - and
    // so the sweep - unchanged
    std::vector<uint32_t> crs, lbs;
    if (h->cl_feasible) {
        const uint32_t C = (uint32_t)h->cl_size;
        uint32_t slice = 1;
        for (const GroupDesc& g : gdesc) slice = std::max(slice, (g.nv + C - 1) / C);
        h->cl_slice = slice;
        h->cl_lcap = 1;
        h->cl_phase_max = 0;
        std::vector<uint32_t> tmp;
        for (GroupDesc& g : gdesc) {
            const uint32_t crs_base = (uint32_t)crs.size(), lb_base = (uint32_t)lbs.size();
            std::vector<uint32_t> owned(C, 0);
            for (uint32_t col = 0; col < g.n_col; ++col) {
                const uint32_t b = gcol_start[g.col_base + col], e = gcol_start[g.col_base + col + 1];
                std::vector<std::vector<uint32_t>> by(C);
                std::vector<uint32_t> maj(e - b);
                std::vector<int32_t> lean(e - b);   // vertices in the next slice minus in the previous one
                std::vector<uint32_t> cnt(C, 0);
                for (uint32_t k = b; k < e; ++k) {
                    const uint32_t* q = &h->tets[4ull * h->tet_order[k]];
                    uint32_t r[4], best = 0, bestn = 0;
                    for (int i = 0; i < 4; ++i) r[i] = (old_to_new[q[i]] - g.v0) / slice;
                    for (int i = 0; i < 4; ++i) {
                        uint32_t n = 0;
                        for (int j = 0; j < 4; ++j) n += r[j] == r[i];
                        if (n > bestn || (n == bestn && r[i] < best)) { best = r[i]; bestn = n; }
                    }
                    int32_t l = 0;
                    for (int i = 0; i < 4; ++i) l += (r[i] == best + 1) - (r[i] + 1 == best);
                    maj[k - b] = best;
                    lean[k - b] = l;
                    cnt[best]++;
                }
                const uint64_t n_col_tets = e - b;
                const uint32_t maj_max = *std::max_element(cnt.begin(), cnt.end());
                const uint32_t even_max = (uint32_t)((n_col_tets + C - 1) / C);
                std::vector<uint32_t> owner_of(maj);
                if (maj_max > std::max<uint32_t>(256u, (even_max + 31) / 32 * 32)) {
                    std::vector<uint32_t> idx(e - b);
                    std::iota(idx.begin(), idx.end(), 0u);
                    std::stable_sort(idx.begin(), idx.end(), [&](uint32_t x, uint32_t y) {
                        return maj[x] != maj[y] ? maj[x] < maj[y] : lean[x] < lean[y];
                    });
                    for (uint32_t rr = 0; rr < C; ++rr)
                        for (uint64_t q = n_col_tets * rr / C; q < n_col_tets * (rr + 1) / C; ++q)
                            owner_of[idx[q]] = rr;
                }
                for (uint32_t k = b; k < e; ++k) by[owner_of[k - b]].push_back(h->tet_order[k]);
                uint32_t k = b;
                for (uint32_t rr = 0; rr < C; ++rr) {
                    crs.push_back(k);
                    lbs.push_back(owned[rr]);
                    owned[rr] += (uint32_t)by[rr].size();
                    h->cl_phase_max = std::max(h->cl_phase_max, (uint32_t)by[rr].size());
                    for (uint32_t t : by[rr]) h->tet_order[k++] = t;
                }
            }
            crs.push_back(g.n_col ? gcol_start[g.col_base + g.n_col] : 0);
            for (uint32_t rr = 0; rr < C; ++rr) h->cl_lcap = std::max(h->cl_lcap, owned[rr]);
            g.col_base = crs_base;
            g.lb_base = lb_base;
        }
        const size_t need = cluster_smem_bytes(h->cl_slice, P, h->prm.body_contacts ? 1 : 0, h->cl_lcap);
        const int blk = h->prm.block_size ? std::min(h->prm.block_size, kClusterMaxBlock) : 256;
        int active = 0;
        const bool ok = need <= (size_t)smem_optin && cluster_configure(blk, need) == cudaSuccess &&
                        cluster_max_active(h->cl_size, blk, need, &active) == cudaSuccess && active >= 1;
        if (!ok) {
            cudaGetLastError();
            if (need > (size_t)smem_optin - 4096 && shrink_tries < 4) {
                ++shrink_tries;
                cap_slice = (uint32_t)((double)cap_slice * (double)(smem_optin - 4096) / (double)need * 0.97);
                goto plan_again;
            }
            if (h->prm.exec_mode == SBS_EXEC_CLUSTER)
                return fail(h, SBS_EINVAL, "scene does not fit the cluster-resident mode");
            allow_cluster = false;
            goto plan_again;
        }
    }
    // 4. block size
    h->block = h->prm.block_size ? h->prm.block_size : 256;
    int tail_thr = h->prm.tail_threshold >= 0 ? h->prm.tail_threshold : h->block;
    h->first_tail = h->global_modes ? (uint32_t)K : 0;
    while (h->global_modes && h->first_tail > 0 &&
           h->colour_offsets[h->first_tail] - h->colour_offsets[h->first_tail - 1] <= (uint32_t)tail_thr)
        --h->first_tail;
    // 6. per-vertex data in library order
    h->inv_mass.assign(V, 0.0f);
    h->is_kin.assign(V, 0);
    std::vector<float4> xw(V), vel(V), accv;
    bool need_acc = h->has_acc || !h->groups.empty();
    if (need_acc) accv.assign(V, make_float4(0, 0, 0, 0));
    for (uint32_t n = 0; n < V; ++n) {
        uint32_t o = new_to_old[n];
        double m = h->mass[o];
        float w = m > 0.0 ? (float)(1.0 / m) : 0.0f;
        h->inv_mass[n] = w;
        xw[n] = make_float4((float)h->xinit[3ull * o], (float)h->xinit[3ull * o + 1], (float)h->xinit[3ull * o + 2], w);
        vel[n] = make_float4(h->vinit[3ull * o], h->vinit[3ull * o + 1], h->vinit[3ull * o + 2], 0.0f);
        if (h->kin_group[o] >= 0) {
            const KinGroup& g = h->groups[h->kin_group[o]];
            vel[n].w = (float)(1 + h->kin_group[o]);
            h->is_kin[n] = 1;
            accv[n] = make_float4((float)(h->x0[3ull * o] - g.cx), (float)(h->x0[3ull * o + 1] - g.cy),
                                  (float)(h->x0[3ull * o + 2] - g.cz), 0.0f);
        } else if (h->has_acc) {
            accv[n] = make_float4(h->acc[3ull * o], h->acc[3ull * o + 1], h->acc[3ull * o + 2], 0.0f);
        }
    }
    // 7. per-tet data in slot order
    std::vector<uint4> tid(T);
    std::vector<float4> d0(T), d1(T), d2(T);
    for (uint32_t k = 0; k < T; ++k) {
        uint32_t t = h->tet_order[k];
        const uint32_t* q = &h->tets[4ull * t];
        double D[3][3], Di[3][3], det;
        for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) D[r][c] = h->x0[3ull * q[c] + r] - h->x0[3ull * q[3] + r];
        invert3(D, Di, &det);
        const double V0 = det / 6.0;
        tid[k] = make_uint4(old_to_new[q[0]], old_to_new[q[1]], old_to_new[q[2]], old_to_new[q[3]]);
        d0[k] = make_float4((float)Di[0][0], (float)Di[0][1], (float)Di[0][2], (float)V0);
        d1[k] = make_float4((float)Di[1][0], (float)Di[1][1], (float)Di[1][2], (float)h->tet_mu[t]);
        d2[k] = make_float4((float)Di[2][0], (float)Di[2][1], (float)Di[2][2], (float)h->tet_lam[t]);
    }
    // 8. surface vertices: faces (topology.cpp:335-342) with != 2 incident tets
    {
        std::unordered_map<uint64_t, uint32_t> fc;
        fc.reserve(4ull * T);
        for (uint32_t t = 0; t < T; ++t) {
            const uint32_t* q = &h->tets[4ull * t];
            const uint32_t fl[4][3] = {{q[0], q[1], q[3]}, {q[1], q[2], q[3]}, {q[2], q[0], q[3]}, {q[0], q[2], q[1]}};
            for (auto& f : fl) {
                uint32_t s3[3] = {f[0], f[1], f[2]};
                std::sort(s3, s3 + 3);
                uint64_t key = ((uint64_t)s3[0] * V + s3[1]) * (uint64_t)V + s3[2];
                fc[key]++;
            }
        }
        std::vector<uint8_t> on(V, 0);
        for (auto& kv : fc) {
            if (kv.second == 2) continue;
            uint64_t key = kv.first;
            uint32_t c = (uint32_t)(key % V);
            key /= V;
            uint32_t b = (uint32_t)(key % V);
            uint32_t a = (uint32_t)(key / V);
            on[old_to_new[a]] = on[old_to_new[b]] = on[old_to_new[c]] = 1;
        }
        h->surf.clear();
        for (uint32_t n = 0; n < V; ++n)
            if (on[n]) h->surf.push_back(n);
        // boundary faces per tet slot (spatial hash queries and contact faces)
        h->bmask.assign(T, 0);
        for (uint32_t k = 0; k < T; ++k) {
            const uint32_t* q = &h->tets[4ull * h->tet_order[k]];
            const uint32_t fl[4][3] = {{q[0], q[1], q[3]}, {q[1], q[2], q[3]}, {q[2], q[0], q[3]}, {q[0], q[2], q[1]}};
            for (int f = 0; f < 4; ++f) {
                uint32_t s3[3] = {fl[f][0], fl[f][1], fl[f][2]};
                std::sort(s3, s3 + 3);
                if (fc[((uint64_t)s3[0] * V + s3[1]) * (uint64_t)V + s3[2]] == 1) h->bmask[k] |= (uint8_t)(1u << f);
            }
        }
        // visual models (tetrahedral_mesh_boundary.cpp:76-120): the mesh lists
        // each distinct face once, at its first appearance over tets in input
        // order and faces_copy order, with that appearance's winding; boundary
        // faces are those with != 2 incident tets; surface vertices are
        // numbered by first appearance in the boundary triangles
        h->vis_tri0.assign(1, 0);
        h->vis_sv0.assign(1, 0);
        h->vis_tris.clear();
        h->vis_map.clear();
        std::unordered_map<uint64_t, uint8_t> emitted;
        for (const BodyHost& b : h->bodies) {
            std::unordered_map<uint32_t, uint32_t> local;
            for (uint32_t t = b.t0; t < b.t0 + b.nt; ++t) {
                const uint32_t* q = &h->tets[4ull * t];
                const uint32_t fl[4][3] = {{q[0], q[1], q[3]}, {q[1], q[2], q[3]}, {q[2], q[0], q[3]}, {q[0], q[2], q[1]}};
                for (auto& f : fl) {
                    uint32_t s3[3] = {f[0], f[1], f[2]};
                    std::sort(s3, s3 + 3);
                    const uint64_t key = ((uint64_t)s3[0] * V + s3[1]) * (uint64_t)V + s3[2];
                    if (fc[key] == 2 || !emitted.emplace(key, 1).second) continue;
                    for (int j = 0; j < 3; ++j) {
                        auto it = local.find(f[j]);
                        if (it == local.end()) {
                            it = local.emplace(f[j], (uint32_t)(h->vis_map.size() - h->vis_sv0.back())).first;
                            h->vis_map.push_back(f[j] - b.v0);
                        }
                        h->vis_tris.push_back(it->second);
                    }
                }
            }
            h->vis_tri0.push_back((uint32_t)(h->vis_tris.size() / 3));
            h->vis_sv0.push_back((uint32_t)h->vis_map.size());
        }
    }
    // 9. device allocations and upload
    SceneDev& d = h->d;
    d.n_verts = V;
    d.wait_ns = h->prm.wait_limit_us > 0 ? 1000ull * (unsigned long long)h->prm.wait_limit_us : 2000000000ull;
    d.n_tets = T;
    d.n_surf = (uint32_t)h->surf.size();
    d.n_kin = 0;
    sbs_status s;
#define AL(p, n) if ((s = dalloc(h, &(p), (n))) != SBS_OK) return s
    AL(d.xi, V); AL(d.xn, V); AL(d.v, V);
    if (need_acc) { AL(d.acc, V); } else d.acc = nullptr;
    AL(d.model, T); AL(d.tet, T); AL(d.dm0, T); AL(d.dm1, T); AL(d.dm2, T); AL(d.lam0, T); AL(d.lam1, T);
    AL(d.surf, d.n_surf);
    // kMaxPlanes ground-contact segments, then the body-contact segment
    const size_t ncont = (size_t)(kMaxPlanes + 1) * d.n_surf;
    AL(d.contacts, ncont); AL(d.contact_lam, ncont);
    AL(d.counters, 16);
    AL(d.time, 1); AL(d.err, 1); AL(d.bar, 2);
    AL(d.red_out, 4);
    AL(d.partials, 6 * 4096);
#undef AL
    d.kin_vert = nullptr;
    d.kin_rel = nullptr;
    d.body_contact_cap = 0;
    // distance constraints in colour order, ends in library vertex slots
    d.n_edges = (uint32_t)h->dist_p.size();
    d.edge = nullptr;
    d.edge_p = nullptr;
    d.edge_lam = nullptr;
    if (d.n_edges) {
        const int KE = colour_edges(h->dist_v, V, h->edge_order, h->edge_offsets);
        if (KE < 0 || KE > kMaxEdgeColours)
            return fail(h, SBS_ECOLOUR, "distance constraints need more than 64 colours");
        std::vector<uint2> ev(d.n_edges);
        std::vector<float4> ep(d.n_edges);
        for (uint32_t k = 0; k < d.n_edges; ++k) {
            const uint32_t e = h->edge_order[k];
            ev[k] = make_uint2(old_to_new[h->dist_v[2ull * e]], old_to_new[h->dist_v[2ull * e + 1]]);
            ep[k] = h->dist_p[e];
        }
        if ((s = dalloc(h, &d.edge, d.n_edges)) != SBS_OK) return s;
        if ((s = dalloc(h, &d.edge_p, d.n_edges)) != SBS_OK) return s;
        if ((s = dalloc(h, &d.edge_lam, d.n_edges)) != SBS_OK) return s;
        if ((s = upload(h, d.edge, ev.data(), ev.size() * sizeof(uint2))) != SBS_OK) return s;
        if ((s = upload(h, d.edge_p, ep.data(), ep.size() * sizeof(float4))) != SBS_OK) return s;
        CU(h, cudaMemsetAsync(d.edge_lam, 0, d.n_edges * sizeof(float), h->st));
    }
    if ((s = upload(h, d.xi, xw.data(), V * sizeof(float4))) != SBS_OK) return s;
    if ((s = upload(h, d.xn, xw.data(), V * sizeof(float4))) != SBS_OK) return s;
    if ((s = upload(h, d.v, vel.data(), V * sizeof(float4))) != SBS_OK) return s;
    if (need_acc && (s = upload(h, d.acc, accv.data(), V * sizeof(float4))) != SBS_OK) return s;
    if ((s = upload(h, d.tet, tid.data(), T * sizeof(uint4))) != SBS_OK) return s;
    if ((s = upload(h, d.dm0, d0.data(), T * sizeof(float4))) != SBS_OK) return s;
    if ((s = upload(h, d.dm1, d1.data(), T * sizeof(float4))) != SBS_OK) return s;
    if ((s = upload(h, d.dm2, d2.data(), T * sizeof(float4))) != SBS_OK) return s;
    {
        std::vector<uint8_t> mdl(T);
        for (uint32_t k = 0; k < T; ++k) mdl[k] = (uint8_t)h->tet_model[h->tet_order[k]];
        if ((s = upload(h, d.model, mdl.data(), T)) != SBS_OK) return s;
    }
    if ((s = upload(h, d.surf, h->surf.data(), d.n_surf * sizeof(uint32_t))) != SBS_OK) return s;
    {
        // visual models on the device: slots, triangle corners, incidence
        SurfaceDev& sd = h->sd;
        sd.n_sv = (uint32_t)h->vis_map.size();
        sd.n_tri = (uint32_t)(h->vis_tris.size() / 3);
        std::vector<uint32_t> slot(sd.n_sv), cnt(sd.n_sv + 1, 0), inc(3ull * sd.n_tri);
        std::vector<uint4> tri(sd.n_tri);
        for (size_t b = 0; b < h->bodies.size(); ++b) {
            const uint32_t v0 = h->bodies[b].v0, sv0 = h->vis_sv0[b];
            for (uint32_t i = sv0; i < h->vis_sv0[b + 1]; ++i) slot[i] = old_to_new[v0 + h->vis_map[i]];
            for (uint32_t k = h->vis_tri0[b]; k < h->vis_tri0[b + 1]; ++k) {
                const uint32_t* c = &h->vis_tris[3ull * k];
                tri[k] = make_uint4(slot[sv0 + c[0]], slot[sv0 + c[1]], slot[sv0 + c[2]], 0u);
                for (int j = 0; j < 3; ++j) cnt[sv0 + c[j] + 1]++;
            }
        }
        for (uint32_t i = 0; i < sd.n_sv; ++i) cnt[i + 1] += cnt[i];
        std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
        for (size_t b = 0; b < h->bodies.size(); ++b)
            for (uint32_t k = h->vis_tri0[b]; k < h->vis_tri0[b + 1]; ++k)
                for (int j = 0; j < 3; ++j) inc[fill[h->vis_sv0[b] + h->vis_tris[3ull * k + j]]++] = k;
        if ((s = dalloc(h, &sd.slot, sd.n_sv)) != SBS_OK) return s;
        if ((s = dalloc(h, &sd.inc_start, sd.n_sv + 1)) != SBS_OK) return s;
        if ((s = dalloc(h, &sd.inc, 3ull * sd.n_tri)) != SBS_OK) return s;
        if ((s = dalloc(h, &sd.tri, sd.n_tri)) != SBS_OK) return s;
        if ((s = dalloc(h, &sd.normal, sd.n_sv)) != SBS_OK) return s;
        if ((s = dalloc(h, &sd.stage, 6ull * sd.n_sv)) != SBS_OK) return s;
        if ((s = upload(h, sd.slot, slot.data(), slot.size() * 4)) != SBS_OK) return s;
        if ((s = upload(h, sd.inc_start, cnt.data(), cnt.size() * 4)) != SBS_OK) return s;
        if ((s = upload(h, sd.inc, inc.data(), inc.size() * 4)) != SBS_OK) return s;
        if ((s = upload(h, sd.tri, tri.data(), tri.size() * sizeof(uint4))) != SBS_OK) return s;
        // the body constructor's update_visual_model (tetrahedral_body.cpp:25)
        CU(h, cudaMemsetAsync(sd.normal, 0, sd.n_sv * sizeof(float4), h->st));
        CU(h, launch_surface_update(sd, d.xn, 0, sd.n_sv, 1, nullptr, 6, h->st));
        CU(h, cudaStreamSynchronize(h->st));   // host vectors above go out of scope
    }
    CU(h, cudaMemsetAsync(d.lam0, 0, T * sizeof(float), h->st));
    CU(h, cudaMemsetAsync(d.lam1, 0, T * sizeof(float), h->st));
    CU(h, cudaMemsetAsync(d.counters, 0, 16 * sizeof(uint32_t), h->st));
    CU(h, cudaMemsetAsync(d.time, 0, sizeof(double), h->st));
    CU(h, cudaMemsetAsync(d.err, 0, sizeof(int), h->st));
    CU(h, cudaMemsetAsync(d.bar, 0, 2 * sizeof(unsigned), h->st));
    if ((s = dalloc(h, &h->d_o2n, V)) != SBS_OK) return s;
    if ((s = dalloc(h, &h->d_stage_x, 3ull * V)) != SBS_OK) return s;
    if ((s = dalloc(h, &h->d_stage_v, 3ull * V)) != SBS_OK) return s;
    if ((s = dalloc(h, &h->d_bad, 1)) != SBS_OK) return s;
    if ((s = upload(h, h->d_o2n, old_to_new.data(), V * sizeof(uint32_t))) != SBS_OK) return s;
    // spatial hash for body-body contacts
    if (h->prm.body_contacts && d.n_surf > 0) {
        HashDev& hd = h->hd;
        double cell = h->prm.hash_cell;
        if (!(cell > 0)) {  // 2 x mean edge length of the rest meshes
            double sum = 0;
            uint64_t cnt = 0;
            static const int E[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
            for (uint32_t t = 0; t < T; ++t)
                for (auto& e : E) {
                    const uint32_t a = h->tets[4ull * t + e[0]], b = h->tets[4ull * t + e[1]];
                    double l2 = 0;
                    for (int k = 0; k < 3; ++k) {
                        const double dd = h->x0[3ull * a + k] - h->x0[3ull * b + k];
                        l2 += dd * dd;
                    }
                    sum += std::sqrt(l2);
                    ++cnt;
                }
            cell = 2.0 * sum / (double)cnt;
        }
        h->hash_cell = cell;
        hd.inv_h = (float)(1.0 / cell);
        hd.depth = (float)cell;
        hd.self = h->prm.body_contacts == 2 ? 1 : 0;
        uint32_t cap = 1024;
        while (cap < 2 * d.n_surf) cap *= 2;
        if (cap > (1u << 22)) return fail(h, SBS_EINVAL, "too many surface vertices for the contact hash");
        hd.mask = cap - 1;
        std::vector<uint32_t> vb(V), qlist;
        for (uint32_t bi = 0; bi < h->bodies.size(); ++bi)
            for (uint32_t i = 0; i < h->bodies[bi].nv; ++i) vb[h->bodies[bi].v0 + i] = bi;
        for (uint32_t k = 0; k < T; ++k)
            if (h->bmask[k]) qlist.push_back(k);
        hd.n_query = (uint32_t)qlist.size();
        const uint32_t tiles = (cap + 1023) / 1024;
        if ((s = dalloc(h, &hd.keys, cap)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.count, cap)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.start, cap)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.fill, cap)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.tile_sums, tiles)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.tile_scan, tiles)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.tile_sums2, 8)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.tile_scan2, 8)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.vslot, d.n_surf)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.entries, d.n_surf)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.vbody, V)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.bmask, T)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.query, qlist.size())) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.best, V)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.bc_q, V)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.bc_n, V)) != SBS_OK) return s;
        if ((s = dalloc(h, &hd.n_cand, 1)) != SBS_OK) return s;
        hd.cand = nullptr;
        hd.cand_cap = h->prm.candidate_capacity;
        if (hd.cand_cap && (s = dalloc(h, &hd.cand, hd.cand_cap)) != SBS_OK) return s;
        if ((s = upload(h, hd.vbody, vb.data(), V * 4)) != SBS_OK) return s;
        if ((s = upload(h, hd.bmask, h->bmask.data(), T)) != SBS_OK) return s;
        if ((s = upload(h, hd.query, qlist.data(), qlist.size() * 4)) != SBS_OK) return s;
        CU(h, cudaMemsetAsync(hd.bc_q, 0, V * sizeof(float4), h->st));
        CU(h, cudaMemsetAsync(hd.bc_n, 0, V * sizeof(float4), h->st));
        CU(h, cudaMemsetAsync(hd.n_cand, 0, sizeof(unsigned long long), h->st));
        h->body_on = true;
    }
    // cluster-resident mode: packed (rank, slice offset) vertex ids, surface
    // flags, group descriptors and per-group colour tables
    if (h->cl_feasible) {
        ClusterDev& c = h->cd;
        c.cluster_size = (uint32_t)h->cl_size;
        uint32_t slice = 1;
        slice = h->cl_slice;
        c.slice = slice;
        c.xn_minus_xi = slice * 16u;
        c.n_groups = (uint32_t)gdesc.size();
        h->cl_smem = cluster_smem_bytes(slice, P, h->body_on ? 1 : 0, h->cl_lcap);
        c.stage = 0;
        if (h->prm.stage_records) {
            // staging buffers for the largest (colour, CTA) tet set, when the
            // cluster still launches with them
            const size_t staged = cluster_smem_bytes(slice, P, h->body_on ? 1 : 0, h->cl_lcap, h->cl_phase_max);
            const int blk = h->prm.block_size ? std::min(h->prm.block_size, kClusterMaxBlock) : 256;
            int active = 0;
            if (staged + 2048 <= (size_t)smem_optin && cluster_configure(blk, staged) == cudaSuccess &&
                cluster_max_active(h->cl_size, blk, staged, &active) == cudaSuccess && active >= 1) {
                c.stage = h->cl_phase_max;
                h->cl_smem = staged;
            }
            cudaGetLastError();
        }
        c.lcap = h->cl_lcap;
        c.body = h->body_on ? 1 : 0;
        c.bc_q = h->hd.bc_q;
        c.bc_n = h->hd.bc_n;
        std::vector<uint32_t> vgroup(V);
        for (uint32_t gi = 0; gi < gdesc.size(); ++gi)
            for (uint32_t n = gdesc[gi].v0; n < gdesc[gi].v0 + gdesc[gi].nv; ++n) vgroup[n] = gi;
        auto pack = [&](uint32_t n) {
            const uint32_t local = n - gdesc[vgroup[n]].v0;
            return ((local / slice) << 24) | (local % slice);
        };
        std::vector<uint4> tp(T);
        for (uint32_t k = 0; k < T; ++k) {
            tp[k] = make_uint4(pack(tid[k].x), pack(tid[k].y), pack(tid[k].z), pack(tid[k].w));
            if (h->tet_model[h->tet_order[k]] != SBS_MODEL_STVK) tp[k].x |= 0x80000000u;
        }
        std::vector<uint8_t> vf(V, 0);
        for (uint32_t n : h->surf) vf[n] = 1;
        if ((s = dalloc(h, &c.tet_packed, T)) != SBS_OK) return s;
        if ((s = dalloc(h, &c.vflags, V)) != SBS_OK) return s;
        if ((s = dalloc(h, &c.groups, gdesc.size())) != SBS_OK) return s;
        if ((s = dalloc(h, &c.col_start, crs.size())) != SBS_OK) return s;
        if ((s = dalloc(h, &c.lam_base, lbs.size())) != SBS_OK) return s;
        if ((s = upload(h, c.tet_packed, tp.data(), T * sizeof(uint4))) != SBS_OK) return s;
        if ((s = upload(h, c.vflags, vf.data(), V)) != SBS_OK) return s;
        if ((s = upload(h, c.groups, gdesc.data(), gdesc.size() * sizeof(GroupDesc))) != SBS_OK) return s;
        if ((s = upload(h, c.col_start, crs.data(), crs.size() * 4)) != SBS_OK) return s;
        if ((s = upload(h, c.lam_base, lbs.data(), lbs.size() * 4)) != SBS_OK) return s;
        if ((size_t)smem_optin < h->cl_smem + 2048) h->cl_feasible = false;
    }
    CU(h, cudaStreamSynchronize(h->st));
    // 10. step constants
    StepParams& p = h->base;
    std::memset(&p, 0, sizeof(p));
    p.gx = (float)h->prm.gravity[0];
    p.gy = (float)h->prm.gravity[1];
    p.gz = (float)h->prm.gravity[2];
    p.gravity_mode = h->prm.gravity_mode;
    p.n_colours = K;
    p.first_tail = (int)h->first_tail;
    p.n_analytic = (int)h->planes.size();
    p.n_planes = (int)(h->planes.size() + h->grids.size());
    for (size_t i = 0; i < h->planes.size(); ++i) p.planes[i] = h->planes[i];
    h->grid_dev.assign(h->grids.size(), nullptr);
    for (size_t g = 0; g < h->grids.size(); ++g) {
        const auto& gh = h->grids[g];
        if ((s = dalloc(h, &h->grid_dev[g], gh.v.size())) != SBS_OK) return s;
        if ((s = upload(h, h->grid_dev[g], gh.v.data(), gh.v.size() * sizeof(float))) != SBS_OK) return s;
        SdfGrid& dg = p.grids[g];
        dg.v = h->grid_dev[g];
        dg.nx = gh.n[0]; dg.ny = gh.n[1]; dg.nz = gh.n[2];
        dg.ox = (float)gh.o[0]; dg.oy = (float)gh.o[1]; dg.oz = (float)gh.o[2];
        dg.hx = (float)gh.h[0]; dg.hy = (float)gh.h[1]; dg.hz = (float)gh.h[2];
        dg.cubic = gh.cubic;
    }
    p.n_kin_groups = (int)h->groups.size();
    p.has_acc = h->has_acc ? 1 : 0;
    p.body_contacts = h->body_on ? 1 : 0;
    for (size_t i = 0; i < h->groups.size(); ++i) p.kin[i] = h->groups[i];
    p.n_edge_colours = d.n_edges ? (int)h->edge_offsets.size() - 1 : 0;
    for (int c = 0; c <= p.n_edge_colours && d.n_edges; ++c) p.edge_start[c] = h->edge_offsets[c];
    if (h->global_modes) {
        p.n_colours = K;
        for (int c = 0; c <= K; ++c) p.colour_start[c] = h->colour_offsets[c];
        for (int c = 0; c < K; ++c) p.colour_split[c] = split[c];
    } else {
        p.n_colours = 0;
        p.first_tail = 0;
    }
    // 11. execution mode
    int occ = 0;
    CU(h, persistent_occupancy(h->block, &occ, h->prm.stage_records >= 2));
    uint32_t maxc = 0;
    for (uint32_t c = 0; c + 1 < h->colour_offsets.size(); ++c)
        maxc = std::max(maxc, h->colour_offsets[c + 1] - h->colour_offsets[c]);
    h->grid = std::max(1, std::min(h->n_sm * 8, (int)((maxc + 31) / 32)));
    int cps = h->prm.ctas_per_sm > 0 ? std::min(h->prm.ctas_per_sm, occ) : occ;
    h->pers_block = h->block;
    h->pers_grid = std::max(1, std::min(cps * h->n_sm, (int)((maxc + 31) / 32)));
    if (h->cl_feasible) {
        h->cl_block = h->prm.block_size ? std::min(h->prm.block_size, kClusterMaxBlock) : 256;
        CU(h, cluster_configure(h->cl_block, h->cl_smem));
        int active = 0;
        cudaError_t e = cluster_max_active(h->cl_size, h->cl_block, h->cl_smem, &active);
        if (e != cudaSuccess || active < 1) {
            cudaGetLastError();
            h->cl_feasible = false;
        } else {
            h->cl_grid = std::max(1, std::min(active, (int)h->cd.n_groups));
        }
    }
    // wavefront mode (only when asked for: measured slower than the grid
    // barrier on every workload - 22.1 vs 8.0 ms on the 98k-tet beam, 34.0 vs
    // 22.1 ms on the 2.6M-tet block, 16.1 vs 13.5 ms on 512 boxes: a CTA of
    // the block polls 22 neighbours on average (36 at most), and each phase
    // pays the release of its stores, the polls' L2 round trips and a fence)
    h->d.prog = nullptr;
    h->d.nb_start = nullptr;
    h->d.nb = nullptr;
    h->d.wave_start = nullptr;
    h->d.wave_idx = nullptr;
    h->wave_grid = 0;
    if (h->global_modes && h->prm.exec_mode == SBS_EXEC_WAVEFRONT) {
        int wocc = 0;
        if (wavefront_occupancy(256, &wocc) == cudaSuccess && wocc > 0) {
            const int G = wocc * h->n_sm;
            std::vector<uint32_t> st_, nb_, ws_, wi_;
            wave_partition(tid, h->colour_offsets, K, G, V, ws_, wi_, st_, nb_);
            if ((s = dalloc(h, &h->d.wave_start, ws_.size())) != SBS_OK) return s;
            if ((s = dalloc(h, &h->d.wave_idx, wi_.size())) != SBS_OK) return s;
            if ((s = upload(h, h->d.wave_start, ws_.data(), ws_.size() * 4)) != SBS_OK) return s;
            if ((s = upload(h, h->d.wave_idx, wi_.data(), wi_.size() * 4)) != SBS_OK) return s;
            if ((s = dalloc(h, &h->d.prog, G)) != SBS_OK) return s;
            if ((s = dalloc(h, &h->d.nb_start, G + 1)) != SBS_OK) return s;
            if ((s = dalloc(h, &h->d.nb, nb_.size())) != SBS_OK) return s;
            if ((s = upload(h, h->d.nb_start, st_.data(), st_.size() * 4)) != SBS_OK) return s;
            if ((s = upload(h, h->d.nb, nb_.data(), nb_.size() * 4)) != SBS_OK) return s;
            CU(h, cudaStreamSynchronize(h->st));
            h->wave_grid = G;
            h->wave_max_nb = 0;
            for (int b = 0; b < G; ++b) h->wave_max_nb = std::max(h->wave_max_nb, st_[b + 1] - st_[b]);
        }
        cudaGetLastError();
    }
    if (h->prm.exec_mode == SBS_EXEC_WAVEFRONT && !h->wave_grid)
        return fail(h, SBS_EINVAL, "scene does not run in the wavefront mode");
    if (!h->global_modes && !h->cl_feasible) return fail(h, SBS_ESTATE, "no execution mode fits this scene");
    if (h->prm.exec_mode == SBS_EXEC_CLUSTER && !h->cl_feasible)
        return fail(h, SBS_EINVAL, "scene does not fit the cluster-resident mode");
    if (h->prm.exec_mode == SBS_EXEC_AUTO)
        h->exec_mode = h->cl_feasible ? SBS_EXEC_CLUSTER : SBS_EXEC_PERSISTENT;
    else
        h->exec_mode = h->prm.exec_mode;
    if (h->exec_mode == SBS_EXEC_PERSISTENT && occ < 1) h->exec_mode = SBS_EXEC_GRAPH;
    h->tuned = h->prm.exec_mode != SBS_EXEC_AUTO;
    h->finalized = true;
    return SBS_OK;
}

static sbs_status check_ready(sbs_gpu* h) {
    if (!h) return SBS_EINVAL;
    if (!h->finalized) return fail(h, SBS_ESTATE, "call before finalize");
    return SBS_OK;
}

static sbs_status check_err(sbs_gpu* h) {
    int e = 0;
    CU(h, cudaMemcpyAsync(&e, h->d.err, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    if (e != 0) {
        // reported once: the flag is cleared so that later frames run (the
        // frame that set it stopped early and is left incomplete)
        CU(h, cudaMemsetAsync(h->d.err, 0, sizeof(int), h->st));
        CU(h, cudaStreamSynchronize(h->st));
        return fail(h, (sbs_status)e, "device reported an error (code " + std::to_string(e) + ")");
    }
    return SBS_OK;
}

// Enqueues one frame in graph mode (per-phase kernels).  Used both for
// capture and for direct launches.
static sbs_status enqueue_frame_kernels(sbs_gpu* h, const StepParams& p) {
    const SceneDev& d = h->d;
    cudaStream_t st = h->st;
    CU(h, cudaMemsetAsync(d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), st));
    CU(h, launch_detect_ground(d, p, st));
    if (h->body_on) CU(h, launch_body_detect(d, h->hd, st));
    for (int sub = 0; sub < p.substeps; ++sub) {
        CU(h, launch_predict(d, p, sub, st));
        for (int it = 0; it < p.iterations; ++it) {
            CU(h, launch_contacts(d, p, it == 0, st));
            CU(h, launch_body_contacts(d, p, it == 0, st));
            for (int c = 0; c < p.first_tail; ++c) CU(h, launch_colour(d, p, c, it == 0, h->block, h->grid, st));
            CU(h, launch_tail(d, p, it == 0, h->block, st));
            for (int c = 0; c < p.n_edge_colours; ++c) CU(h, launch_edges(d, p, c, it == 0, st));
        }
        CU(h, launch_finalize(d, p, st));
    }
    CU(h, launch_end_frame(d, st));
    return SBS_OK;
}

static sbs_status enqueue_warm_init(sbs_gpu* h, const StepParams& p);
static sbs_status enqueue_segments(sbs_gpu* h, const StepParams& p, uint32_t iterations, bool reset,
                                   cudaStream_t st);

// Learned warm start: per substep predict -> features -> MLP -> carry or fit
// sweeps, then the sweeps continue from those multipliers.
// In the cluster mode the sweeps of each substep run as one launch of the
// cluster-resident kernel on the warm-started positions and multipliers
// (kClExternal | kClCarry); the other modes enqueue the per-phase kernels.
static sbs_status enqueue_warm_frame(sbs_gpu* h, const StepParams& p, uint32_t substeps, uint32_t iterations) {
    CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
    CU(h, launch_detect_ground(h->d, p, h->st));
    if (h->body_on) CU(h, launch_body_detect(h->d, h->hd, h->st));
    for (uint32_t sub = 0; sub < substeps; ++sub) {
        CU(h, launch_predict(h->d, p, (int)sub, h->st));
        sbs_status s = enqueue_warm_init(h, p);
        if (s) return s;
        if (h->exec_mode == SBS_EXEC_CLUSTER) {
            StepParams q = p;
            q.substeps = 1;
            q.cl_flags = kClExternal | kClCarry;
            CU(h, launch_cluster_frame(h->d, h->cd, q, h->sim_time, h->cl_grid, h->cl_block, h->cl_smem, h->st));
        } else if ((s = enqueue_segments(h, p, iterations, false, h->st)) != SBS_OK) {
            return s;
        }
        CU(h, launch_finalize(h->d, p, h->st));
    }
    CU(h, launch_end_frame(h->d, h->st));
    return SBS_OK;
}

// Plain-solver judge (sbs_gpu_set_warm_judge).  A judged warm-started
// substep runs, all on the device:
//   predict; the plain start's residual (predicted positions, zero
//   multipliers); the warm start (features, network, carry or fit); its
//   residual, which keeps the warm start only if it is below the plain
//   start's and otherwise restores the plain start (k_judge_fallback); then
//   a WHILE conditional graph node whose body runs `chunk` sweeps and the
//   residual, until the residual is at or below the target (the residual of
//   a plain substep with the full sweep count, recorded by calibration
//   frames) or the next chunk would pass the cap; velocity update.
// The loop's condition is set by k_residual_final (JudgeOp), on the device,
// so a frame is one graph launch with no host round trip.

// One sweep chunk of the running substep on stream `st`.
static sbs_status enqueue_judge_chunk(sbs_gpu* h, const StepParams& p, cudaStream_t st) {
    if (h->exec_mode == SBS_EXEC_CLUSTER) {
        StepParams q = p;
        q.substeps = 1;
        q.iterations = (int)h->judge_chunk;
        q.cl_flags = kClExternal | kClCarry | kClContinue;
        CU(h, launch_cluster_frame(h->d, h->cd, q, h->sim_time, h->cl_grid, h->cl_block, h->cl_smem, st));
        return SBS_OK;
    }
    return enqueue_segments(h, p, h->judge_chunk, false, st);
}

static sbs_status enqueue_judge_residual(sbs_gpu* h, const StepParams& p, int zero_lam, const JudgeOp& op,
                                         cudaStream_t st) {
    const int grid = std::max(1, std::min(4096, (int)((h->n_tets + 255) / 256)));
    CU(h, launch_residual_ex(h->d, p, 256, grid, 0, st, zero_lam, &op));
    return SBS_OK;
}

// The sweep loop of substep `sub` inside the frame graph being captured on
// h->st: a conditional handle (set by the start residual's judge step), the
// WHILE node, and its body captured on the side stream.
static sbs_status enqueue_judge_loop(sbs_gpu* h, const StepParams& p, int sub) {
    cudaStreamCaptureStatus cs;
    cudaGraph_t g = nullptr;
    CU(h, cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &g, nullptr, nullptr, nullptr));
    if (cs != cudaStreamCaptureStatusActive || !g) return fail(h, SBS_ESTATE, "judged frames run as graphs");
    cudaGraphConditionalHandle hc;
    CU(h, cudaGraphConditionalHandleCreate(&hc, g, 0, 0));
    JudgeOp op{};
    op.kind = kJudgeStart;
    op.substep = sub;
    op.chunk = h->judge_chunk;
    op.cap = h->judge_cap ? h->judge_cap : (uint32_t)p.iterations;
    op.j = h->d_judge;
    op.cond = (unsigned long long)hc;
    sbs_status s = enqueue_judge_residual(h, p, 0, op, h->st);
    if (s) return s;
    CU(h, launch_judge_fallback(h->d, h->wd, h->d_judge, h->st));
    const cudaGraphNode_t* deps = nullptr;
    const cudaGraphEdgeData* edges = nullptr;
    size_t nd = 0;
    CU(h, cudaStreamGetCaptureInfo(h->st, &cs, nullptr, &g, &deps, &edges, &nd));
    cudaGraphNodeParams np{};
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = hc;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    CU(h, cudaGraphAddNode(&node, g, deps, edges, nd, &np));
    cudaGraph_t body = np.conditional.phGraph_out[0];
    CU(h, cudaStreamBeginCaptureToGraph(h->side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    op.kind = kJudgeChunk;
    s = enqueue_judge_chunk(h, p, h->side);
    if (s == SBS_OK) s = enqueue_judge_residual(h, p, 0, op, h->side);
    cudaGraph_t body_out = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->side, &body_out);
    if (s) return s;
    if (e != cudaSuccess) return fail(h, SBS_ECUDA, std::string("loop body capture: ") + cudaGetErrorString(e));
    CU(h, cudaStreamUpdateCaptureDependencies(h->st, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
    CU(h, launch_judge_end(h->d_judge, sub, h->st));
    return SBS_OK;
}

static sbs_status enqueue_judged_frame(sbs_gpu* h, const StepParams& p, uint32_t substeps, uint32_t iterations,
                                       bool calibrate) {
    if (calibrate && h->exec_mode == SBS_EXEC_CLUSTER && h->cl_grid == 1 && h->cd.n_groups == 1) {
        // one cluster holds the scene: the plain frame kernel itself records
        // each substep's final residual and prediction (kClCalibrate)
        StepParams q = p;
        q.cl_flags = kClCalibrate;
        q.judge = h->d_judge;
        q.judge_xpred = h->wd.xpred;
        CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
        if (h->body_on) CU(h, launch_body_detect(h->d, h->hd, h->st));
        CU(h, launch_cluster_frame(h->d, h->cd, q, h->sim_time, h->cl_grid, h->cl_block, h->cl_smem, h->st));
        CU(h, launch_end_frame(h->d, h->st));
        double t_end = h->sim_time;
        for (uint32_t k = 0; k < substeps; ++k) t_end += p.dt_d;
        CU(h, launch_store_time(h->d.time, t_end, h->st));
        return SBS_OK;
    }
    CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
    CU(h, launch_detect_ground(h->d, p, h->st));
    if (h->body_on) CU(h, launch_body_detect(h->d, h->hd, h->st));
    for (uint32_t sub = 0; sub < substeps; ++sub) {
        CU(h, launch_predict(h->d, p, (int)sub, h->st));
        sbs_status s;
        if (calibrate) {
            // a plain substep (the features only record the prediction for
            // the next warm substep's previous-displacement feature)
            CU(h, launch_features(h->d, h->wd, p, h->xpred_valid ? 1 : 0, h->st));
            h->xpred_valid = true;
            CU(h, cudaMemsetAsync(h->d.contact_lam, 0, (size_t)(kMaxPlanes + 1) * h->d.n_surf * sizeof(float),
                                  h->st));
            if (h->exec_mode == SBS_EXEC_CLUSTER) {
                StepParams q = p;
                q.substeps = 1;
                q.cl_flags = kClExternal;
                CU(h, launch_cluster_frame(h->d, h->cd, q, h->sim_time, h->cl_grid, h->cl_block, h->cl_smem,
                                           h->st));
            } else if ((s = enqueue_segments(h, p, iterations, true, h->st)) != SBS_OK) {
                return s;
            }
            JudgeOp op{};
            op.kind = kJudgeCalib;
            op.substep = (int)sub;
            op.j = h->d_judge;
            if ((s = enqueue_judge_residual(h, p, 0, op, h->st)) != SBS_OK) return s;
        } else {
            JudgeOp op{};
            op.kind = kJudgePlain0;
            op.substep = (int)sub;
            op.j = h->d_judge;
            if ((s = enqueue_judge_residual(h, p, 1, op, h->st)) != SBS_OK) return s;
            if ((s = enqueue_warm_init(h, p)) != SBS_OK) return s;
            if (h->exec_mode == SBS_EXEC_CLUSTER && h->cl_grid == 1 && h->cd.n_groups == 1) {
                // one cluster holds the whole scene: the judge runs inside its
                // kernel, one launch per substep (residual checks reduced
                // across the cluster's shared memory)
                StepParams q = p;
                q.substeps = 1;
                q.cl_flags = kClExternal | kClCarry | kClJudge;
                q.judge = h->d_judge;
                q.judge_xpred = h->wd.xpred;
                q.judge_chunk = h->judge_chunk;
                q.judge_cap = h->judge_cap ? h->judge_cap : (uint32_t)p.iterations;
                q.judge_substep = (int)sub;
                CU(h, launch_cluster_frame(h->d, h->cd, q, h->sim_time, h->cl_grid, h->cl_block, h->cl_smem, h->st));
            } else if ((s = enqueue_judge_loop(h, p, (int)sub)) != SBS_OK) {
                return s;
            }
        }
        CU(h, launch_finalize(h->d, p, h->st));
    }
    CU(h, launch_end_frame(h->d, h->st));
    return SBS_OK;
}

// Launches the CUDA graph of `key`, capturing it from `enqueue` first.
static sbs_status run_graph(sbs_gpu* h, const GraphKey& key, const std::function<sbs_status()>& enqueue) {
    auto it = h->graphs.find(key);
    if (it == h->graphs.end()) {
        cudaGraph_t g;
        const uint64_t k0 = launch_counter();
        CU(h, cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
        sbs_status s = enqueue();
        cudaError_t e = cudaStreamEndCapture(h->st, &g);
        h->graph_kernels[key] = launch_counter() - k0;
        launch_counter() = k0;   // captured, not run
        if (s != SBS_OK) return s;
        if (e != cudaSuccess) return fail(h, SBS_ECUDA, std::string("capture: ") + cudaGetErrorString(e));
        cudaGraphExec_t ge;
        e = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return fail(h, SBS_ECUDA, std::string("instantiate: ") + cudaGetErrorString(e));
        it = h->graphs.emplace(key, ge).first;
    }
    CU(h, cudaGraphLaunch(it->second, h->st));
    count_launch(h->graph_kernels[key]);
    return SBS_OK;
}

static sbs_status run_frame(sbs_gpu* h, double dt, uint32_t substeps, uint32_t iterations) {
    StepParams p;
    fill_params(h, p, dt, substeps, iterations);
    double t_end = h->sim_time;
    for (uint32_t k = 0; k < substeps; ++k) t_end += dt;   // same double sequence as the CPU loop
    const uint64_t launches0 = launch_counter();
    if (h->mlp && h->judge_chunk) {
        // judged warm-started frame, or a calibration frame of plain
        // substeps when no target is known yet or one is due
        if (substeps > (uint32_t)kMaxJudgeSubsteps)
            return fail(h, SBS_EINVAL, "judged frames take at most 64 substeps");
        const bool calibrate = !h->judge_target_valid ||
                               (h->judge_calib_every > 0 && h->judged_frames % h->judge_calib_every == 0);
        sbs_status s;
        if (calibrate && h->exec_mode == SBS_EXEC_CLUSTER && h->cl_grid == 1 && h->cd.n_groups == 1) {
            // one launch of the frame kernel, which takes the frame's start
            // time as a parameter: launched directly, like the plain frame
            s = enqueue_judged_frame(h, p, substeps, iterations, true);
        } else {
            const GraphKey key{dt, substeps, iterations, calibrate ? 3 : (h->xpred_valid ? 2 : 1)};
            s = run_graph(h, key, [&]() { return enqueue_judged_frame(h, p, substeps, iterations, calibrate); });
        }
        if (s) return s;
        h->xpred_valid = true;
        h->judged_frames++;
        if (calibrate) h->judge_target_valid = true;
    } else if (h->mlp) {
        // the warm-started frame as one CUDA graph per shape (a substep is
        // hundreds of small kernels); whether the previous substep's
        // displacement is known at the frame's start is part of the shape
        const GraphKey key{dt, substeps, iterations, h->xpred_valid ? 2 : 1};
        sbs_status s = run_graph(h, key, [&]() { return enqueue_warm_frame(h, p, substeps, iterations); });
        if (s) return s;
        h->xpred_valid = true;
    } else if (h->exec_mode == SBS_EXEC_CLUSTER) {
        // the kernel publishes the frame's contacts into the last-frame slots
        CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
        if (h->body_on) CU(h, launch_body_detect(h->d, h->hd, h->st));
        CU(h, launch_cluster_frame(h->d, h->cd, p, h->sim_time, h->cl_grid, h->cl_block, h->cl_smem, h->st));
        CU(h, launch_end_frame(h->d, h->st));
        CU(h, launch_store_time(h->d.time, t_end, h->st));
    } else if (h->exec_mode == SBS_EXEC_WAVEFRONT) {
        if (h->contacts_live)
            CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
        if (h->body_on) CU(h, launch_body_detect(h->d, h->hd, h->st));
        CU(h, cudaMemsetAsync(h->d.bar, 0, 2 * sizeof(unsigned), h->st));
        CU(h, cudaMemsetAsync(h->d.prog, 0, h->wave_grid * sizeof(uint32_t), h->st));
        CU(h, launch_wavefront_frame(h->d, p, 256, h->wave_grid, h->st));
    } else if (h->exec_mode == SBS_EXEC_PERSISTENT) {
        // the frame kernel expects zero live contact counters (it zeroes them
        // itself at frame end); a standalone detect or a frame stopped by an
        // error may have left them set
        CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
        if (h->body_on) CU(h, launch_body_detect(h->d, h->hd, h->st));
        CU(h, cudaMemsetAsync(h->d.bar, 0, 2 * sizeof(unsigned), h->st));   // barrier arrival count
        if (h->withhold_arrival) {
            // one arrival short: 0xFFFFFFFF + gridDim arrivals wraps to gridDim - 1
            CU(h, cudaMemsetAsync(h->d.bar, 0xFF, sizeof(unsigned), h->st));
            h->withhold_arrival = false;
        }
        CU(h, launch_persistent_frame(h->d, p, h->pers_block, h->pers_grid, h->st, h->prm.stage_records >= 2));
    } else {
        const GraphKey key{dt, substeps, iterations, 0};
        sbs_status s = run_graph(h, key, [&]() { return enqueue_frame_kernels(h, p); });
        if (s) return s;
    }
    h->kernel_launches += launch_counter() - launches0;
    h->frames++;
    h->projections += (uint64_t)substeps * iterations * h->n_tets;
    h->contacts_live = false;
    h->sim_time = t_end;
    if (!h->mlp) h->xpred_valid = false;   // a plain frame does not record its predictions
    return SBS_OK;
}

// Drops the captured frame graphs (they hold the step parameters).
static void clear_graphs(sbs_gpu* h) {
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    h->graphs.clear();
    h->graph_kernels.clear();
}

// Autotuner: times each candidate configuration on a copy of the state and
// restores the state afterwards.
static sbs_status autotune_modes(sbs_gpu* h, double dt, uint32_t substeps, uint32_t iterations);

// The execution mode is chosen by timing plain frames, also when a warm
// start is attached (its graphs are rebuilt for the chosen mode).
static sbs_status autotune(sbs_gpu* h, double dt, uint32_t substeps, uint32_t iterations) {
    sbs_mlp* m = h->mlp;
    const bool xv = h->xpred_valid;
    h->mlp = nullptr;
    sbs_status s = autotune_modes(h, dt, substeps, iterations);
    h->mlp = m;
    h->xpred_valid = xv;   // the tuner restores the state it stepped
    clear_graphs(h);
    return s;
}

static sbs_status autotune_modes(sbs_gpu* h, double dt, uint32_t substeps, uint32_t iterations) {
    const SceneDev& d = h->d;
    const size_t V = d.n_verts;
    float4 *bxi, *bxn, *bv;
    double* btime;
    CU(h, cudaMalloc((void**)&bxi, V * sizeof(float4)));
    CU(h, cudaMalloc((void**)&bxn, V * sizeof(float4)));
    CU(h, cudaMalloc((void**)&bv, V * sizeof(float4)));
    CU(h, cudaMalloc((void**)&btime, sizeof(double)));
    CU(h, cudaMemcpyAsync(bxi, d.xi, V * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
    CU(h, cudaMemcpyAsync(bxn, d.xn, V * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
    CU(h, cudaMemcpyAsync(bv, d.v, V * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
    CU(h, cudaMemcpyAsync(btime, d.time, sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    struct Cand { int mode, block, grid; };
    std::vector<Cand> cands;
    uint32_t maxc = 0;
    for (uint32_t c = 0; c < h->n_colours; ++c)
        maxc = std::max(maxc, h->colour_offsets[c + 1] - h->colour_offsets[c]);
    const int need = std::max(1, (int)((maxc + 31) / 32));
    if (h->cl_feasible)
        for (int blk : {256, 320, 384, 512}) cands.push_back({SBS_EXEC_CLUSTER, blk, 0});
    for (int blk : {128, 256, 512}) {
        if (!h->global_modes) break;
        int occ = 0;
        if (persistent_occupancy(blk, &occ, h->prm.stage_records >= 2) != cudaSuccess || occ < 1) continue;
        for (int g : {h->n_sm / 2, h->n_sm, 2 * h->n_sm, occ * h->n_sm}) {
            int gg = std::max(1, std::min({g, occ * h->n_sm, need}));
            bool dup = false;
            for (auto& c : cands) dup |= (c.mode == SBS_EXEC_PERSISTENT && c.block == blk && c.grid == gg);
            if (!dup) cands.push_back({SBS_EXEC_PERSISTENT, blk, gg});
        }
    }
    if (h->global_modes) cands.push_back({SBS_EXEC_GRAPH, 256, h->grid});
    const int saved_mode = h->exec_mode, saved_pb = h->pers_block, saved_pg = h->pers_grid;
    const uint64_t saved_frames = h->frames, saved_proj = h->projections;
    const double saved_time = h->sim_time;
    float best = 1e30f;
    Cand bestc{saved_mode, h->exec_mode == SBS_EXEC_CLUSTER ? h->cl_block : saved_pb, saved_pg};
    for (const Cand& c : cands) {
        h->exec_mode = c.mode;
        if (c.mode == SBS_EXEC_PERSISTENT) { h->pers_block = c.block; h->pers_grid = c.grid; }
        if (c.mode == SBS_EXEC_CLUSTER) {
            int active = 0;
            if (cluster_configure(c.block, h->cl_smem) != cudaSuccess ||
                cluster_max_active(h->cl_size, c.block, h->cl_smem, &active) != cudaSuccess || active < 1) {
                cudaGetLastError();
                continue;
            }
            h->cl_block = c.block;
            h->cl_grid = std::max(1, std::min(active, (int)h->cd.n_groups));
        }
        sbs_status s = run_frame(h, dt, substeps, iterations);  // warm-up (and graph capture)
        if (s != SBS_OK) continue;
        CU(h, cudaEventRecord(h->ev0, h->st));
        for (int r = 0; r < 3 && s == SBS_OK; ++r) s = run_frame(h, dt, substeps, iterations);
        CU(h, cudaEventRecord(h->ev1, h->st));
        CU(h, cudaEventSynchronize(h->ev1));
        if (s != SBS_OK) continue;
        if (check_err(h) != SBS_OK) break;
        float ms = 0;
        CU(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
        if (ms < best) { best = ms; bestc = c; }
    }
    h->exec_mode = bestc.mode;
    if (bestc.mode == SBS_EXEC_PERSISTENT) { h->pers_block = bestc.block; h->pers_grid = bestc.grid; }
    // second stage, for a winning global mode: the small-colour merge
    // threshold (colours of at most that many tets run one after another in
    // one CTA, saving a grid barrier or a launch each), unless the caller set it
    if ((bestc.mode == SBS_EXEC_PERSISTENT || bestc.mode == SBS_EXEC_GRAPH) && h->prm.tail_threshold < 0 &&
        best < 1e30f) {
        const uint32_t ft0 = h->first_tail;
        uint32_t best_ft = ft0;
        std::vector<uint32_t> tried{ft0};
        for (uint32_t thr : {0u, 256u, 1024u, 4096u}) {
            uint32_t ft = h->n_colours;
            while (ft > 0 && h->colour_offsets[ft] - h->colour_offsets[ft - 1] <= thr) --ft;
            if (std::find(tried.begin(), tried.end(), ft) != tried.end()) continue;
            tried.push_back(ft);
            h->first_tail = ft;
            h->base.first_tail = (int)ft;
            clear_graphs(h);
            sbs_status s = run_frame(h, dt, substeps, iterations);
            if (s != SBS_OK) continue;
            CU(h, cudaEventRecord(h->ev0, h->st));
            for (int r = 0; r < 3 && s == SBS_OK; ++r) s = run_frame(h, dt, substeps, iterations);
            CU(h, cudaEventRecord(h->ev1, h->st));
            CU(h, cudaEventSynchronize(h->ev1));
            if (s != SBS_OK) continue;
            if (check_err(h) != SBS_OK) break;
            float ms = 0;
            CU(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
            if (ms < best) { best = ms; best_ft = ft; }
        }
        h->first_tail = best_ft;
        h->base.first_tail = (int)best_ft;
        clear_graphs(h);
    }
    if (bestc.mode == SBS_EXEC_CLUSTER) {
        int active = 0;
        h->cl_block = bestc.block;
        CU(h, cluster_configure(h->cl_block, h->cl_smem));
        CU(h, cluster_max_active(h->cl_size, h->cl_block, h->cl_smem, &active));
        h->cl_grid = std::max(1, std::min(active, (int)h->cd.n_groups));
    }
    h->frames = saved_frames;
    h->projections = saved_proj;
    h->sim_time = saved_time;
    CU(h, cudaMemcpyAsync(d.xi, bxi, V * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
    CU(h, cudaMemcpyAsync(d.xn, bxn, V * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
    CU(h, cudaMemcpyAsync(d.v, bv, V * sizeof(float4), cudaMemcpyDeviceToDevice, h->st));
    CU(h, cudaMemcpyAsync(d.time, btime, sizeof(double), cudaMemcpyDeviceToDevice, h->st));
    CU(h, cudaMemsetAsync(d.counters, 0, 16 * sizeof(uint32_t), h->st));
    CU(h, cudaStreamSynchronize(h->st));
    cudaFree(bxi); cudaFree(bxn); cudaFree(bv); cudaFree(btime);
    h->tuned = true;
    (void)saved_pb; (void)saved_pg;
    return check_err(h);
}

sbs_status sbs_gpu_step(sbs_gpu* h, double frame_dt, uint32_t substeps, uint32_t iterations) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!(frame_dt > 0) || substeps == 0 || substeps > 1000 || iterations > 100000)
        return fail(h, SBS_EINVAL, "step: bad frame_dt/substeps/iterations");
    const double dt = frame_dt / (double)substeps;
    if (!h->tuned) {
        s = autotune(h, dt, substeps, iterations);
        if (s) return s;
    }
    return run_frame(h, dt, substeps, iterations);
}

sbs_status sbs_gpu_step_timed(sbs_gpu* h, double frame_dt, uint32_t substeps, uint32_t iterations) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!h->tuned) {
        s = sbs_gpu_step(h, frame_dt, substeps, iterations);  // tunes, then steps
        if (s) return s;
        CU(h, cudaStreamSynchronize(h->st));
        return check_err(h);
    }
    CU(h, cudaEventRecord(h->ev0, h->st));
    s = sbs_gpu_step(h, frame_dt, substeps, iterations);
    if (s) return s;
    CU(h, cudaEventRecord(h->ev1, h->st));
    CU(h, cudaEventSynchronize(h->ev1));
    float ms = 0;
    CU(h, cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    h->last_frame_ms = ms;
    return check_err(h);
}

sbs_status sbs_gpu_withhold_barrier_arrival(sbs_gpu* h) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (h->exec_mode != SBS_EXEC_PERSISTENT || h->mlp)
        return fail(h, SBS_ESTATE, "withhold_barrier_arrival: the handle does not run persistent frames");
    h->withhold_arrival = true;
    return SBS_OK;
}

sbs_status sbs_gpu_detect_contacts(sbs_gpu* h) {
    sbs_status s = check_ready(h);
    if (s) return s;
    StepParams p;
    fill_params(h, p, 1.0, 1, 1);
    CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
    CU(h, launch_detect_ground(h->d, p, h->st));
    if (h->body_on) CU(h, launch_body_detect(h->d, h->hd, h->st));
    h->contacts_live = true;
    return SBS_OK;
}

sbs_status sbs_gpu_predict(sbs_gpu* h, double dt) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!(dt > 0)) return fail(h, SBS_EINVAL, "dt");
    StepParams p;
    fill_params(h, p, dt, 1, 1);
    CU(h, launch_predict(h->d, p, 0, h->st));
    return SBS_OK;
}

sbs_status sbs_gpu_update_velocities(sbs_gpu* h, double dt) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!(dt > 0)) return fail(h, SBS_EINVAL, "dt");
    StepParams p;
    fill_params(h, p, dt, 1, 1);
    CU(h, launch_finalize(h->d, p, h->st));
    h->sim_time += dt;
    return SBS_OK;
}

sbs_status sbs_gpu_solve(sbs_gpu* h, double dt, uint32_t iterations) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!(dt > 0)) return fail(h, SBS_EINVAL, "dt");
    StepParams p;
    fill_params(h, p, dt, 1, iterations);
    if (!h->contacts_live) CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
    // one launch per vertex-disjoint colour segment (all groups' colours in
    // sweep order), whatever the execution mode of sbs_gpu_step
    if ((s = enqueue_segments(h, p, iterations, true, h->st)) != SBS_OK) return s;
    h->projections += (uint64_t)iterations * h->n_tets;
    return SBS_OK;
}

sbs_status sbs_gpu_residual(sbs_gpu* h, double dt, double* residual, double* energy) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!(dt > 0)) return fail(h, SBS_EINVAL, "dt");
    StepParams p;
    fill_params(h, p, dt, 1, 1);
    const int grid = std::max(1, std::min(4096, (int)((h->n_tets + 255) / 256)));
    CU(h, launch_residual_ex(h->d, p, 256, grid, h->contacts_live ? 0 : kMaxPlanes + 1, h->st));
    double out[4];
    CU(h, cudaMemcpyAsync(out, h->d.red_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    s = check_err(h);
    if (s) return s;
    h->residual = std::sqrt(std::max(0.0, out[0] + out[2]));
    h->energy = out[1];
    if (residual) *residual = h->residual;
    if (energy) *energy = h->energy;
    return SBS_OK;
}

static sbs_status body_range(sbs_gpu* h, int32_t body, const BodyHost** b) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (body < 0 || body >= (int32_t)h->bodies.size()) return fail(h, SBS_EINVAL, "body id");
    *b = &h->bodies[body];
    return SBS_OK;
}

// body >= 0: one body; body == -1: the whole scene in global vertex order
static sbs_status state_range(sbs_gpu* h, int32_t body, const BodyHost** b) {
    if (body != -1) return body_range(h, body, b);
    sbs_status s = check_ready(h);
    if (s) return s;
    *b = &h->all_bodies;
    return SBS_OK;
}

// Device -> caller: gather in input order on the device, one copy back.
static sbs_status read_fields(sbs_gpu* h, int32_t body, const float4* xsrc, float* xout, const float4* vsrc,
                              float* vout) {
    const BodyHost* b;
    sbs_status s = state_range(h, body, &b);
    if (s) return s;
    const size_t bytes = 3ull * b->nv * sizeof(float);
    int bad = 0;
    CU(h, cudaMemsetAsync(h->d_bad, 0, sizeof(int), h->st));
    if (vout) {
        CU(h, launch_gather_xyz(vsrc, h->d_o2n, b->v0, b->nv, h->d_stage_v, 0, h->d_bad, h->st));
        CU(h, cudaMemcpyAsync(vout, h->d_stage_v, bytes, cudaMemcpyDeviceToHost, h->st));
    }
    if (xout) {
        CU(h, launch_gather_xyz(xsrc, h->d_o2n, b->v0, b->nv, h->d_stage_x, 1, h->d_bad, h->st));
        CU(h, cudaMemcpyAsync(xout, h->d_stage_x, bytes, cudaMemcpyDeviceToHost, h->st));
    }
    CU(h, cudaMemcpyAsync(&bad, h->d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    s = check_err(h);
    if (s) return s;
    if (bad && h->prm.check_finite) return fail(h, SBS_ENAN, "non-finite positions");
    return SBS_OK;
}

sbs_status sbs_gpu_get_state(sbs_gpu* h, int32_t body, float* x, float* v) {
    if (!h) return SBS_EINVAL;
    return read_fields(h, body, h->d.xn, x, h->d.v, v);
}

sbs_status sbs_gpu_get_predicted(sbs_gpu* h, int32_t body, float* xi) {
    if (!h || !xi) return fail(h, SBS_EINVAL, "null");
    return read_fields(h, body, h->d.xi, xi, nullptr, nullptr);
}

// Caller -> device: one copy in, checked for finite positions on the device,
// scattered into the library's layout (.w of each record kept).
static sbs_status write_fields(sbs_gpu* h, int32_t body, const float* x, bool both, const float* v) {
    const BodyHost* b;
    sbs_status s = state_range(h, body, &b);
    if (s) return s;
    const size_t bytes = 3ull * b->nv * sizeof(float);
    // One synchronisation at the end: the staging buffers are ordered by the
    // stream, and the scatters skip on the device when the position check
    // failed, so a rejected call leaves the state as it was.
    int bad = 0;
    CU(h, cudaMemsetAsync(h->d_bad, 0, sizeof(int), h->st));
    if (x) {
        CU(h, cudaMemcpyAsync(h->d_stage_x, x, bytes, cudaMemcpyHostToDevice, h->st));
        CU(h, launch_check_finite(h->d_stage_x, 3ull * b->nv, h->d_bad, h->st));
        CU(h, launch_scatter_xyz(h->d.xi, both ? h->d.xn : nullptr, h->d_o2n, b->v0, b->nv, h->d_stage_x, h->st,
                                 h->d_bad));
    }
    if (v) {
        CU(h, cudaMemcpyAsync(h->d_stage_v, v, bytes, cudaMemcpyHostToDevice, h->st));
        CU(h, launch_scatter_xyz(h->d.v, nullptr, h->d_o2n, b->v0, b->nv, h->d_stage_v, h->st, h->d_bad));
    }
    CU(h, cudaMemcpyAsync(&bad, h->d_bad, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    if (bad) return fail(h, SBS_EINVAL, "non-finite input position");
    return SBS_OK;
}

sbs_status sbs_gpu_set_state(sbs_gpu* h, int32_t body, const float* x, const float* v) {
    if (!h) return SBS_EINVAL;
    h->xpred_valid = false;
    return write_fields(h, body, x, true, v);
}

sbs_status sbs_gpu_set_predicted(sbs_gpu* h, int32_t body, const float* xi) {
    if (!h || !xi) return fail(h, SBS_EINVAL, "null");
    h->xpred_valid = false;
    return write_fields(h, body, xi, false, nullptr);
}

sbs_status sbs_gpu_get_tet_order(sbs_gpu* h, uint32_t* order, uint32_t* offsets, uint32_t cap_offsets,
                                 uint32_t* n_colours) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (n_colours) *n_colours = h->n_colours;
    if (order) std::copy(h->tet_order.begin(), h->tet_order.end(), order);
    if (offsets) {
        if (cap_offsets < h->n_colours + 1) return fail(h, SBS_EINVAL, "offsets capacity");
        std::copy(h->colour_offsets.begin(), h->colour_offsets.end(), offsets);
    }
    return SBS_OK;
}

sbs_status sbs_gpu_get_lambdas(sbs_gpu* h, float* lambdas) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!lambdas) return fail(h, SBS_EINVAL, "null");
    std::vector<float> a(h->n_tets), b(h->n_tets);
    CU(h, cudaMemcpyAsync(a.data(), h->d.lam0, h->n_tets * sizeof(float), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaMemcpyAsync(b.data(), h->d.lam1, h->n_tets * sizeof(float), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    for (uint32_t k = 0; k < h->n_tets; ++k) {
        lambdas[2ull * h->tet_order[k]] = a[k];
        lambdas[2ull * h->tet_order[k] + 1] = b[k];
    }
    return check_err(h);
}

sbs_status sbs_gpu_get_distance_order(sbs_gpu* h, uint32_t* order, uint32_t* offsets, uint32_t cap_offsets,
                                      uint32_t* n_colours) {
    sbs_status s = check_ready(h);
    if (s) return s;
    const uint32_t K = h->d.n_edges ? (uint32_t)h->edge_offsets.size() - 1 : 0;
    if (n_colours) *n_colours = K;
    if (order) std::copy(h->edge_order.begin(), h->edge_order.end(), order);
    if (offsets && K) {
        if (cap_offsets < K + 1) return fail(h, SBS_EINVAL, "offsets capacity");
        std::copy(h->edge_offsets.begin(), h->edge_offsets.end(), offsets);
    }
    return SBS_OK;
}

sbs_status sbs_gpu_get_distance_lambdas(sbs_gpu* h, float* lambdas) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!lambdas) return fail(h, SBS_EINVAL, "null");
    const uint32_t E = h->d.n_edges;
    if (!E) return SBS_OK;
    std::vector<float> a(E);
    CU(h, cudaMemcpyAsync(a.data(), h->d.edge_lam, E * sizeof(float), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    for (uint32_t k = 0; k < E; ++k) lambdas[h->edge_order[k]] = a[k];
    return check_err(h);
}

// library vertex id -> global id in add order
static uint32_t to_global(const sbs_gpu* h, uint32_t n) {
    // bodies are contiguous; find the body by binary search on v0
    size_t lo = 0, hi = h->bodies.size();
    while (hi - lo > 1) {
        size_t mid = (lo + hi) / 2;
        if (h->bodies[mid].v0 <= n) lo = mid;
        else hi = mid;
    }
    const BodyHost& b = h->bodies[lo];
    return b.v0 + b.new_to_old[n - b.v0];
}

sbs_status sbs_gpu_get_contacts(sbs_gpu* h, uint32_t* verts, float* qn, uint32_t cap, uint32_t* n) {
    sbs_status s = check_ready(h);
    if (s) return s;
    uint32_t cnt[16];
    CU(h, cudaMemcpyAsync(cnt, h->d.counters, sizeof(cnt), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    const uint32_t* c = h->contacts_live ? cnt : cnt + kMaxPlanes + 1;
    std::vector<std::pair<std::pair<uint32_t, uint32_t>, std::array<float, 6>>> all;
    // ground planes in order, then the body-body segment (ordered after them)
    const size_t P = h->planes.size() + h->grids.size();   // environment slots
    for (size_t seg = 0; seg <= P; ++seg) {
        const size_t src = seg < P ? seg : (size_t)kMaxPlanes;
        if (seg == P && !h->body_on) break;
        const uint32_t m = std::min(c[src], h->d.n_surf);
        std::vector<Contact> buf(m);
        if (m)
            CU(h, cudaMemcpyAsync(buf.data(), h->d.contacts + src * h->d.n_surf, m * sizeof(Contact),
                                  cudaMemcpyDeviceToHost, h->st));
        CU(h, cudaStreamSynchronize(h->st));
        for (const Contact& k : buf) {
            uint32_t vid;
            std::memcpy(&vid, &k.q.w, 4);
            all.push_back({{(uint32_t)seg, to_global(h, vid)}, {k.q.x, k.q.y, k.q.z, k.n.x, k.n.y, k.n.z}});
        }
    }
    std::sort(all.begin(), all.end(), [](const auto& a, const auto& b) { return a.first < b.first; });
    if (n) *n = (uint32_t)all.size();
    for (uint32_t i = 0; i < all.size() && i < cap; ++i) {
        if (verts) verts[i] = all[i].first.second;
        if (qn) std::copy(all[i].second.begin(), all[i].second.end(), qn + 6ull * i);
    }
    return check_err(h);
}

sbs_status sbs_gpu_get_candidates(sbs_gpu* h, uint64_t* pairs, uint64_t cap, uint64_t* n) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!h->body_on) return fail(h, SBS_ESTATE, "body contacts are off");
    if (!h->hd.cand) return fail(h, SBS_ESTATE, "candidate recording is off (params.candidate_capacity = 0)");
    unsigned long long total = 0;
    CU(h, cudaMemcpyAsync(&total, h->hd.n_cand, sizeof(total), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    const uint64_t m = std::min<uint64_t>(total, h->hd.cand_cap);
    std::vector<unsigned long long> buf(m);
    if (m) CU(h, cudaMemcpyAsync(buf.data(), h->hd.cand, m * 8, cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    for (auto& k : buf) {
        const uint32_t v = (uint32_t)(k >> 32), slot = (uint32_t)(k & 0xFFFFFFFFull);
        k = ((unsigned long long)to_global(h, v) << 32) | h->tet_order[slot];
    }
    std::sort(buf.begin(), buf.end());
    if (n) *n = total;
    if (pairs)
        for (uint64_t i = 0; i < m && i < cap; ++i) pairs[i] = buf[i];
    return check_err(h);
}

static sbs_status warm_prepare(sbs_gpu* h) {
    if (h->warm_buffers) return SBS_OK;
    const uint32_t V = h->n_verts, T = h->n_tets;
    std::vector<uint32_t> cnt(V + 1, 0), inc(4ull * T);
    std::vector<uint4> tid(T);
    CU(h, cudaMemcpyAsync(tid.data(), h->d.tet, T * sizeof(uint4), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    for (uint32_t t = 0; t < T; ++t) {
        cnt[tid[t].x + 1]++; cnt[tid[t].y + 1]++; cnt[tid[t].z + 1]++; cnt[tid[t].w + 1]++;
    }
    for (uint32_t v = 0; v < V; ++v) cnt[v + 1] += cnt[v];
    std::vector<uint32_t> fill(cnt.begin(), cnt.end() - 1);
    for (uint32_t t = 0; t < T; ++t) {
        inc[fill[tid[t].x]++] = t; inc[fill[tid[t].y]++] = t; inc[fill[tid[t].z]++] = t; inc[fill[tid[t].w]++] = t;
    }
    sbs_status s;
    if ((s = dalloc(h, &h->wd.feat, 16ull * V)) != SBS_OK) return s;
    if ((s = dalloc(h, &h->wd.delta, 3ull * V)) != SBS_OK) return s;
    if ((s = dalloc(h, &h->wd.xpred, V)) != SBS_OK) return s;
    if ((s = dalloc(h, &h->wd.inc_start, V + 1)) != SBS_OK) return s;
    if ((s = dalloc(h, &h->wd.inc, 4ull * T)) != SBS_OK) return s;
    if ((s = dalloc(h, &h->wd.tet_f, 3ull * T)) != SBS_OK) return s;
    if ((s = upload(h, h->wd.inc_start, cnt.data(), (V + 1) * 4)) != SBS_OK) return s;
    if ((s = upload(h, h->wd.inc, inc.data(), 4ull * T * 4)) != SBS_OK) return s;
    CU(h, cudaStreamSynchronize(h->st));
    h->warm_buffers = true;
    return SBS_OK;
}

sbs_status sbs_gpu_set_warm_start(sbs_gpu* h, sbs_mlp* m, uint32_t fit_sweeps) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (m && fit_sweeps > 16) return fail(h, SBS_EINVAL, "fit_sweeps must be 0..16");
    if (m && m->d.device != h->prm.device) return fail(h, SBS_EINVAL, "MLP lives on another device");
    if (m && (s = warm_prepare(h)) != SBS_OK) return s;
    if (m) CU(h, mlp_reserve(m->d, (int)h->n_verts));
    if (m) CU(h, mlp_tc_configure());
    h->mlp = m;
    if (m) h->fit_sweeps = fit_sweeps;
    clear_graphs(h);
    return SBS_OK;
}

sbs_status sbs_gpu_set_warm_judge(sbs_gpu* h, uint32_t check_every, uint32_t max_sweeps, uint32_t calibrate_every,
                                  double fixed_target) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (check_every > 1000 || max_sweeps > 100000 || !(fixed_target >= 0.0) || !std::isfinite(fixed_target))
        return fail(h, SBS_EINVAL, "set_warm_judge: bad arguments");
    if (check_every && max_sweeps && check_every > max_sweeps)
        return fail(h, SBS_EINVAL, "set_warm_judge: check_every above max_sweeps");
    if (check_every && !h->d_judge) {
        if ((s = dalloc(h, &h->d_judge, 1)) != SBS_OK) return s;
        CU(h, cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking));
    }
    h->judge_chunk = check_every;
    h->judge_cap = max_sweeps;
    h->judge_calib_every = calibrate_every;
    h->judge_fixed_target = fixed_target;
    h->judged_frames = 0;
    h->judge_target_valid = false;
    if (h->d_judge) {
        JudgeDev j{};
        if (check_every && fixed_target > 0.0) {
            for (int k = 0; k < kMaxJudgeSubsteps; ++k) j.target[k] = fixed_target;
            h->judge_target_valid = true;
            h->judge_calib_every = 0;
        }
        CU(h, cudaMemcpyAsync(h->d_judge, &j, sizeof(j), cudaMemcpyHostToDevice, h->st));
        CU(h, cudaStreamSynchronize(h->st));
    }
    clear_graphs(h);
    return SBS_OK;
}

sbs_status sbs_gpu_get_warm_stats(sbs_gpu* h, sbs_gpu_warm_stats* out) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!out) return fail(h, SBS_EINVAL, "null");
    *out = sbs_gpu_warm_stats{};
    if (!h->d_judge) return SBS_OK;
    JudgeDev j;
    CU(h, cudaMemcpyAsync(&j, h->d_judge, sizeof(j), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    out->warm_substeps = j.warm_substeps;
    out->calibration_substeps = j.calib_substeps;
    out->sweeps = j.total_sweeps;
    out->fallbacks = j.fallbacks;
    out->capped = j.capped;
    out->mean_residual_ratio = j.warm_substeps ? j.sum_ratio / (double)j.warm_substeps : 0.0;
    out->max_residual_ratio = j.max_ratio;
    out->last_target = j.target[0];
    out->last_residual = j.r_now;
    return check_err(h);
}

// features -> MLP -> fit sweep (multipliers initialised), on the predicted state
static sbs_status enqueue_warm_init(sbs_gpu* h, const StepParams& p) {
    const bool dprev_valid = h->xpred_valid;
    CU(h, launch_features(h->d, h->wd, p, dprev_valid ? 1 : 0, h->st));
    h->xpred_valid = true;
    CU(h, mlp_infer_tc(h->mlp->d, h->wd.feat, (int)h->n_verts, h->wd.delta, h->d.err, (int)SBS_ETIMEOUT, h->n_sm,
                       h->st));
    if (h->fit_sweeps == 0) {
        // carry start: the multipliers stay as the previous substep left
        // them, unless there is no previous substep of this state
        if (!dprev_valid) {
            CU(h, cudaMemsetAsync(h->d.lam0, 0, (size_t)h->n_tets * sizeof(float), h->st));
            CU(h, cudaMemsetAsync(h->d.lam1, 0, (size_t)h->n_tets * sizeof(float), h->st));
        }
        CU(h, launch_carry(h->d, h->wd, h->st));
    }
    for (uint32_t k = 0; k < h->fit_sweeps; ++k)
        for (size_t c = 0; c + 1 < h->colour_offsets.size(); ++c)
            CU(h, launch_fit_segment(h->d, h->wd, p, h->colour_offsets[c], h->colour_offsets[c + 1], k == 0 ? 1 : 0,
                                     h->st));
    CU(h, cudaMemsetAsync(h->d.contact_lam, 0, (size_t)(kMaxPlanes + 1) * h->d.n_surf * sizeof(float), h->st));
    if (h->d.n_edges) CU(h, cudaMemsetAsync(h->d.edge_lam, 0, h->d.n_edges * sizeof(float), h->st));
    return SBS_OK;
}

sbs_status sbs_gpu_warm_start_init(sbs_gpu* h, double dt) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!h->mlp) return fail(h, SBS_ESTATE, "no warm-start network attached");
    if (!(dt > 0)) return fail(h, SBS_EINVAL, "dt");
    StepParams p;
    fill_params(h, p, dt, 1, 1);
    return enqueue_warm_init(h, p);
}

static sbs_status enqueue_segments(sbs_gpu* h, const StepParams& p, uint32_t iterations, bool reset,
                                   cudaStream_t st) {
    for (uint32_t it = 0; it < iterations; ++it) {
        const int first = (reset && it == 0) ? 1 : 0;
        CU(h, launch_contacts(h->d, p, first, st));
        CU(h, launch_body_contacts(h->d, p, first, st));
        for (size_t c = 0; c + 1 < h->colour_offsets.size(); ++c) {
            StepParams q = p;
            q.n_colours = 1;
            q.first_tail = 1;
            q.colour_start[0] = h->colour_offsets[c];
            q.colour_start[1] = h->colour_offsets[c + 1];
            q.colour_split[0] = h->seg_split[c];
            CU(h, launch_colour(h->d, q, 0, first, h->block, h->grid, st));
        }
        for (int c = 0; c < p.n_edge_colours; ++c) CU(h, launch_edges(h->d, p, c, first, st));
    }
    return SBS_OK;
}

sbs_status sbs_gpu_solve_ex(sbs_gpu* h, double dt, uint32_t iterations, int32_t reset_lambda) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!(dt > 0)) return fail(h, SBS_EINVAL, "dt");
    StepParams p;
    fill_params(h, p, dt, 1, iterations);
    if (!h->contacts_live) CU(h, cudaMemsetAsync(h->d.counters, 0, (kMaxPlanes + 1) * sizeof(uint32_t), h->st));
    if ((s = enqueue_segments(h, p, iterations, reset_lambda != 0, h->st)) != SBS_OK) return s;
    h->projections += (uint64_t)iterations * h->n_tets;
    return SBS_OK;
}

sbs_status sbs_gpu_get_features(sbs_gpu* h, float* feat) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!feat) return fail(h, SBS_EINVAL, "null");
    if ((s = warm_prepare(h)) != SBS_OK) return s;
    StepParams p;
    fill_params(h, p, 1.0, 1, 1);
    CU(h, launch_features(h->d, h->wd, p, h->xpred_valid ? 1 : 0, h->st));
    h->xpred_valid = true;
    std::vector<float> buf(16ull * h->n_verts);
    CU(h, cudaMemcpyAsync(buf.data(), h->wd.feat, buf.size() * 4, cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    for (uint32_t n = 0; n < h->n_verts; ++n)
        std::copy(&buf[16ull * n], &buf[16ull * n + 16], feat + 16ull * to_global(h, n));
    return check_err(h);
}

sbs_status sbs_gpu_get_masses(sbs_gpu* h, float* inv_mass) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!inv_mass) return fail(h, SBS_EINVAL, "null");
    for (uint32_t n = 0; n < h->n_verts; ++n) inv_mass[to_global(h, n)] = h->inv_mass[n];
    return SBS_OK;
}

sbs_status sbs_gpu_get_surface(sbs_gpu* h, uint32_t* verts, uint32_t cap, uint32_t* n) {
    sbs_status s = check_ready(h);
    if (s) return s;
    std::vector<uint32_t> g;
    for (uint32_t v : h->surf) g.push_back(to_global(h, v));
    std::sort(g.begin(), g.end());
    if (n) *n = (uint32_t)g.size();
    if (verts)
        for (uint32_t i = 0; i < g.size() && i < cap; ++i) verts[i] = g[i];
    return SBS_OK;
}

sbs_status sbs_gpu_get_surface_mesh(sbs_gpu* h, int32_t body, uint32_t* triangles, uint32_t cap_triangles,
                                    uint32_t* n_triangles, uint32_t* vertex_map, uint32_t cap_vertices,
                                    uint32_t* n_vertices) {
    const BodyHost* b;
    sbs_status s = body_range(h, body, &b);
    if (s) return s;
    const uint32_t t0 = h->vis_tri0[body], nt = h->vis_tri0[body + 1] - t0;
    const uint32_t v0 = h->vis_sv0[body], nv = h->vis_sv0[body + 1] - v0;
    if (n_triangles) *n_triangles = nt;
    if (n_vertices) *n_vertices = nv;
    if (triangles) {
        if (cap_triangles < nt) return fail(h, SBS_EINVAL, "triangle capacity");
        std::copy(&h->vis_tris[3ull * t0], &h->vis_tris[3ull * t0] + 3ull * nt, triangles);
    }
    if (vertex_map) {
        if (cap_vertices < nv) return fail(h, SBS_EINVAL, "vertex capacity");
        std::copy(&h->vis_map[v0], &h->vis_map[v0] + nv, vertex_map);
    }
    return SBS_OK;
}

sbs_status sbs_gpu_update_surface(sbs_gpu* h, int32_t body, int32_t accumulate_normals, float* vertex_buffer,
                                  uint32_t stride) {
    const BodyHost* b;
    sbs_status s = body_range(h, body, &b);
    if (s) return s;
    if (vertex_buffer && stride < 6) return fail(h, SBS_EINVAL, "stride must be >= 6 floats");
    const uint32_t v0 = h->vis_sv0[body], nv = h->vis_sv0[body + 1] - v0;
    bool on_device = false;
    if (vertex_buffer) {
        cudaPointerAttributes attr{};
        CU(h, cudaPointerGetAttributes(&attr, vertex_buffer));
        on_device = attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
        if (on_device && attr.device != h->prm.device) return fail(h, SBS_EINVAL, "buffer lives on another device");
    }
    float* out = !vertex_buffer ? nullptr : on_device ? vertex_buffer : h->sd.stage;
    CU(h, launch_surface_update(h->sd, h->d.xn, v0, nv, accumulate_normals ? 1 : 0, out, on_device ? stride : 6,
                                h->st));
    if (vertex_buffer && !on_device) {
        std::vector<float> buf(6ull * nv);
        CU(h, cudaMemcpyAsync(buf.data(), h->sd.stage, buf.size() * sizeof(float), cudaMemcpyDeviceToHost, h->st));
        CU(h, cudaStreamSynchronize(h->st));
        for (uint32_t i = 0; i < nv; ++i) std::copy(&buf[6ull * i], &buf[6ull * i + 6], vertex_buffer + (size_t)i * stride);
    } else {
        CU(h, cudaStreamSynchronize(h->st));
    }
    return check_err(h);
}

sbs_status sbs_gpu_get_stats(sbs_gpu* h, sbs_gpu_stats* st) {
    sbs_status s = check_ready(h);
    if (s) return s;
    if (!st) return fail(h, SBS_EINVAL, "null");
    std::memset(st, 0, sizeof(*st));
    uint32_t cnt[16];
    CU(h, cudaMemcpyAsync(cnt, h->d.counters, sizeof(cnt), cudaMemcpyDeviceToHost, h->st));
    CU(h, cudaStreamSynchronize(h->st));
    const uint32_t* c = h->contacts_live ? cnt : cnt + kMaxPlanes + 1;
    st->frames = h->frames;
    st->projections = h->projections;
    st->n_vertices = h->n_verts;
    st->n_tets = h->n_tets;
    st->n_colours = h->n_colours;
    st->n_tail_colours = h->n_colours - h->first_tail;
    for (size_t pl = 0; pl < h->planes.size() + h->grids.size(); ++pl) st->n_contacts += c[pl];
    st->n_body_contacts = c[kMaxPlanes];
    st->exec_mode = h->exec_mode;
    st->grid_ctas = h->exec_mode == SBS_EXEC_WAVEFRONT     ? h->wave_grid
                    : h->exec_mode == SBS_EXEC_PERSISTENT ? h->pers_grid
                    : h->exec_mode == SBS_EXEC_CLUSTER  ? h->cl_grid * h->cl_size
                                                        : h->grid;
    st->block_size = h->exec_mode == SBS_EXEC_WAVEFRONT     ? 256
                     : h->exec_mode == SBS_EXEC_PERSISTENT ? h->pers_block
                     : h->exec_mode == SBS_EXEC_CLUSTER  ? h->cl_block
                                                         : h->block;
    st->residual = h->residual;
    st->energy = h->energy;
    st->last_frame_ms = h->last_frame_ms;
    st->kernel_launches = h->kernel_launches;
    st->cluster_phase_max_tets = h->exec_mode == SBS_EXEC_CLUSTER ? h->cl_phase_max : 0;
    return check_err(h);
}

sbs_status sbs_gpu_destroy(sbs_gpu* h) {
    if (!h) return SBS_EINVAL;
    cudaSetDevice(h->prm.device);
    if (h->st) cudaStreamSynchronize(h->st);
    for (auto& kv : h->graphs) cudaGraphExecDestroy(kv.second);
    for (void* p : h->allocations) cudaFree(p);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->st) cudaStreamDestroy(h->st);
    if (h->side) cudaStreamDestroy(h->side);
    delete h;
    return SBS_OK;
}

}  // extern "C"
