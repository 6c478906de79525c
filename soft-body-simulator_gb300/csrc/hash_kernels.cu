// Spatial-hash broad phase and vertex-in-tet narrow phase for body-body (and
// optional self) contacts, run once per frame on the frame-start positions.
//
// Cells: c = floor(x * inv_h) per axis, x and inv_h float, product rounded
// to nearest (__fmul_rn), so the CPU oracle computes the same cells.  The
// 63-bit key packs the three 21-bit biased coordinates exactly (no hash
// collisions between cells).  Surface vertices are inserted into an
// open-addressing table (linear probing, capacity >= 2x entries), counted per
// cell, and laid out contiguously by an exclusive scan of the counts.  Every
// tet with at least one boundary face visits the cells of its AABB; a
// (surface vertex, tet) pair is a candidate when the vertex is not one of the
// tet's vertices and belongs to another body (or self contacts are on).
// Narrow phase (vertex-triangle): the vertex lies behind one of the tet's
// boundary triangles by less than the cell size and projects inside it; the
// contact is that triangle's half-space, frozen for the frame: q = x - d n,
// outward unit normal n (collision_constraint_t form,
// src/physics/xpbd/collision_constraint.cpp:11-19).  One contact per vertex:
// largest d, ties to the lower (sweep slot, face), selected with a 64-bit
// atomicMax (order independent, hence deterministic).
#include <cuda_runtime.h>
#include <stdint.h>

#include "hash_internal.cuh"
#include "launch_count.cuh"
#include "xpbd_internal.cuh"
#include "xpbd_math.cuh"

namespace sbs {

constexpr unsigned long long kEmptyKey = ~0ull;

__device__ __forceinline__ int32_t cell_of(float x, float inv_h) { return (int32_t)floorf(__fmul_rn(x, inv_h)); }

__device__ __forceinline__ unsigned long long cell_key(int32_t cx, int32_t cy, int32_t cz) {
    const unsigned long long m = (1ull << 21) - 1;
    return (((unsigned long long)(uint32_t)(cx + (1 << 20)) & m) << 42) |
           (((unsigned long long)(uint32_t)(cy + (1 << 20)) & m) << 21) |
           ((unsigned long long)(uint32_t)(cz + (1 << 20)) & m);
}

__device__ __forceinline__ uint32_t key_slot(unsigned long long k, uint32_t mask) {
    // splitmix64 finaliser
    k ^= k >> 30;
    k *= 0xbf58476d1ce4e5b9ull;
    k ^= k >> 27;
    k *= 0x94d049bb133111ebull;
    k ^= k >> 31;
    return (uint32_t)k & mask;
}

// Slot of key k (inserting it if absent).
__device__ __forceinline__ uint32_t table_insert(unsigned long long* keys, uint32_t mask, unsigned long long k) {
    uint32_t s = key_slot(k, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long old = atomicCAS(keys + s, kEmptyKey, k);
        if (old == kEmptyKey || old == k) return s;
        s = (s + 1) & mask;
    }
    return 0xFFFFFFFFu;  // unreachable: capacity >= 2x entries
}

// Slot of key k, or 0xFFFFFFFF if absent.
__device__ __forceinline__ uint32_t table_find(const unsigned long long* keys, uint32_t mask, unsigned long long k) {
    uint32_t s = key_slot(k, mask);
    for (uint32_t probe = 0; probe <= mask; ++probe) {
        const unsigned long long cur = keys[s];
        if (cur == k) return s;
        if (cur == kEmptyKey) return 0xFFFFFFFFu;
        s = (s + 1) & mask;
    }
    return 0xFFFFFFFFu;
}

__global__ void k_hash_insert(SceneDev s, HashDev hd) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n_surf; i += gridDim.x * blockDim.x) {
        const float4 x = s.xn[s.surf[i]];
        const unsigned long long k =
            cell_key(cell_of(x.x, hd.inv_h), cell_of(x.y, hd.inv_h), cell_of(x.z, hd.inv_h));
        const uint32_t slot = table_insert(hd.keys, hd.mask, k);
        hd.vslot[i] = slot;
        if (slot != 0xFFFFFFFFu) atomicAdd(hd.count + slot, 1u);
    }
}

// Exclusive scan of count[0..n) into start, 1024 elements per CTA.
__global__ void k_scan_tiles(const uint32_t* in, uint32_t* out, uint32_t* sums, uint32_t n) {
    __shared__ uint32_t warp_tot[32];
    const uint32_t i = blockIdx.x * 1024 + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0u;
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = warp_tot[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= (uint32_t)o) t += y;
        }
        warp_tot[lane] = t;
    }
    __syncthreads();
    const uint32_t before = (wid ? warp_tot[wid - 1] : 0u) + x - v;
    if (i < n) out[i] = before;
    if (threadIdx.x == 1023 && sums) sums[blockIdx.x] = warp_tot[31];
}

__global__ void k_scan_add(uint32_t* out, const uint32_t* sums_scanned, uint32_t n) {
    const uint32_t i = blockIdx.x * 1024 + threadIdx.x;
    if (i < n && blockIdx.x > 0) out[i] += sums_scanned[blockIdx.x];
}

__global__ void k_hash_fill(SceneDev s, HashDev hd) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n_surf; i += gridDim.x * blockDim.x) {
        const uint32_t slot = hd.vslot[i];
        if (slot == 0xFFFFFFFFu) continue;
        const uint32_t pos = hd.start[slot] + atomicAdd(hd.fill + slot, 1u);
        hd.entries[pos] = s.surf[i];
    }
}

// Boundary face f of a tet as a contact plane for point p (faces in
// tetrahedron_t::faces_copy order, src/physics/topology.cpp:335-342): outward
// unit normal n (away from the opposite vertex), signed distance d, and
// whether the projection of p onto the plane falls inside the triangle.
__device__ __forceinline__ bool face_plane(const float4* x, uint4 id, int f, f3 p, float& d, f3& n) {
    const uint32_t v[4] = {id.x, id.y, id.z, id.w};
    const int F[4][4] = {{0, 1, 3, 2}, {1, 2, 3, 0}, {2, 0, 3, 1}, {0, 2, 1, 3}};
    const f3 a = mk(x[v[F[f][0]]]), b = mk(x[v[F[f][1]]]), c = mk(x[v[F[f][2]]]), o = mk(x[v[F[f][3]]]);
    f3 nn = cross(b - a, c - a);
    const float l = sqrtf(dot(nn, nn));
    if (!(l > 0.0f)) return false;
    nn = nn * (1.0f / l);
    if (dot(nn, o - a) > 0.0f) nn = -nn;
    n = nn;
    d = dot(p - a, nn);
    const f3 q = p - nn * d;
    const float ua = dot(nn, cross(b - q, c - q)), ub = dot(nn, cross(c - q, a - q)), uc = dot(nn, cross(a - q, b - q));
    return (ua >= 0.0f && ub >= 0.0f && uc >= 0.0f) || (ua <= 0.0f && ub <= 0.0f && uc <= 0.0f);
}

__device__ __forceinline__ uint32_t orderable(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Narrow phase per candidate: the vertex is behind a boundary triangle of the
// tet by less than the cell size (-h < d < 0) and projects inside it.  Best
// per vertex: largest d, ties to the lower (slot, face), by a 64-bit max of
// (orderable(d) << 32 | ~(slot << 2 | face)).
__global__ void k_hash_query(SceneDev s, HashDev hd) {
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < hd.n_query; q += gridDim.x * blockDim.x) {
        const uint32_t t = hd.query[q];
        const uint4 id = s.tet[t];
        const uint32_t body = hd.vbody[id.x];
        const uint8_t bm = hd.bmask[t];
        const float4 p0 = s.xn[id.x], p1 = s.xn[id.y], p2 = s.xn[id.z], p3 = s.xn[id.w];
        const float lo[3] = {fminf(fminf(p0.x, p1.x), fminf(p2.x, p3.x)), fminf(fminf(p0.y, p1.y), fminf(p2.y, p3.y)),
                             fminf(fminf(p0.z, p1.z), fminf(p2.z, p3.z))};
        const float hi[3] = {fmaxf(fmaxf(p0.x, p1.x), fmaxf(p2.x, p3.x)), fmaxf(fmaxf(p0.y, p1.y), fmaxf(p2.y, p3.y)),
                             fmaxf(fmaxf(p0.z, p1.z), fmaxf(p2.z, p3.z))};
        int32_t c0[3], c1[3];
        for (int a = 0; a < 3; ++a) {
            c0[a] = cell_of(lo[a], hd.inv_h);
            c1[a] = cell_of(hi[a], hd.inv_h);
        }
        for (int32_t cx = c0[0]; cx <= c1[0]; ++cx)
            for (int32_t cy = c0[1]; cy <= c1[1]; ++cy)
                for (int32_t cz = c0[2]; cz <= c1[2]; ++cz) {
                    const uint32_t slot = table_find(hd.keys, hd.mask, cell_key(cx, cy, cz));
                    if (slot == 0xFFFFFFFFu) continue;
                    const uint32_t b = hd.start[slot], e = b + hd.count[slot];
                    for (uint32_t k = b; k < e; ++k) {
                        const uint32_t v = hd.entries[k];
                        if (v == id.x || v == id.y || v == id.z || v == id.w) continue;
                        if (!hd.self && hd.vbody[v] == body) continue;
                        if (hd.cand) {
                            const unsigned long long pos = atomicAdd(hd.n_cand, 1ull);
                            if (pos < hd.cand_cap) hd.cand[pos] = ((unsigned long long)v << 32) | t;
                        } else {
                            atomicAdd(hd.n_cand, 1ull);
                        }
                        const f3 xv = mk(s.xn[v]);
                        for (int f = 0; f < 4; ++f) {
                            if (!((bm >> f) & 1u)) continue;
                            float d;
                            f3 n;
                            if (!face_plane(s.xn, id, f, xv, d, n)) continue;
                            if (!(d < 0.0f && d > -hd.depth)) continue;
                            const unsigned long long packed =
                                ((unsigned long long)orderable(d) << 32) | (uint32_t)(~((t << 2) | (uint32_t)f));
                            atomicMax(hd.best + v, packed);
                        }
                    }
                }
    }
}

// Per surface vertex: turn the best (tet, face) into a contact.  Writes the
// global body-contact segment (graph / persistent modes) and the per-vertex
// records (cluster mode).
__global__ void k_body_contacts(SceneDev s, HashDev hd) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.n_surf; i += gridDim.x * blockDim.x) {
        const uint32_t v = s.surf[i];
        const unsigned long long b = hd.best[v];
        float4 rq = make_float4(0.f, 0.f, 0.f, 0.f), rn = make_float4(0.f, 0.f, 0.f, 0.f);
        if (b != 0ull) {
            const uint32_t key = ~(uint32_t)(b & 0xFFFFFFFFull);
            const uint32_t t = key >> 2;
            const int f = (int)(key & 3u);
            const f3 xv = mk(s.xn[v]);
            float d;
            f3 n;
            face_plane(s.xn, s.tet[t], f, xv, d, n);
            const f3 q = xv - n * d;
            rq = make_float4(q.x, q.y, q.z, 1.0f);
            const uint32_t slot = atomicAdd(&s.counters[kMaxPlanes], 1u);
            rn = make_float4(n.x, n.y, n.z, __uint_as_float(slot));
            if (slot < s.n_surf) {
                Contact c;
                c.q = make_float4(q.x, q.y, q.z, __uint_as_float(v));
                c.n = rn;
                s.contacts[(size_t)kMaxPlanes * s.n_surf + slot] = c;
            }
        }
        hd.bc_q[v] = rq;
        hd.bc_n[v] = rn;
    }
}

static inline int blocks_for(uint32_t n, int cap) {
    long b = ((long)n + 255) / 256;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

cudaError_t launch_body_detect(const SceneDev& s, const HashDev& hd, cudaStream_t st) {
    if (s.n_surf == 0) return cudaSuccess;
    const uint32_t cap = hd.mask + 1;
    cudaError_t e;
    if ((e = cudaMemsetAsync(hd.keys, 0xFF, (size_t)cap * sizeof(unsigned long long), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(hd.count, 0, (size_t)cap * sizeof(uint32_t), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(hd.fill, 0, (size_t)cap * sizeof(uint32_t), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(hd.best, 0, (size_t)s.n_verts * sizeof(unsigned long long), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(hd.n_cand, 0, sizeof(unsigned long long), st)) != cudaSuccess) return e;
    k_hash_insert<<<blocks_for(s.n_surf, 4096), 256, 0, st>>>(s, hd);
    count_launch();
    const uint32_t tiles = (cap + 1023) / 1024;
    k_scan_tiles<<<tiles, 1024, 0, st>>>(hd.count, hd.start, hd.tile_sums, cap);
    count_launch();
    if (tiles > 1) {
        // tiles <= 4096 -> at most 4 levels; the second level fits one CTA for tiles <= 1024
        k_scan_tiles<<<(tiles + 1023) / 1024, 1024, 0, st>>>(hd.tile_sums, hd.tile_scan, hd.tile_sums2, tiles);
        count_launch();
        if (tiles > 1024) {
            k_scan_tiles<<<1, 1024, 0, st>>>(hd.tile_sums2, hd.tile_scan2, nullptr, (tiles + 1023) / 1024);
            count_launch();
            k_scan_add<<<(tiles + 1023) / 1024, 1024, 0, st>>>(hd.tile_scan, hd.tile_scan2, tiles);
            count_launch();
        }
        k_scan_add<<<tiles, 1024, 0, st>>>(hd.start, hd.tile_scan, cap);
        count_launch();
    }
    k_hash_fill<<<blocks_for(s.n_surf, 4096), 256, 0, st>>>(s, hd);
    count_launch();
    if (hd.n_query) {
        k_hash_query<<<blocks_for(hd.n_query, 8192), 256, 0, st>>>(s, hd);
        count_launch();
    }
    k_body_contacts<<<blocks_for(s.n_surf, 4096), 256, 0, st>>>(s, hd);
    count_launch();
    return cudaGetLastError();
}

}  // namespace sbs
