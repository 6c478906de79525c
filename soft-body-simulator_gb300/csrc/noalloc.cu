// Ground-contact detection that allocates no device memory.
//
// Some callers cannot call cudaMalloc at the moment they need contacts: an
// application that owns every device byte through its own allocator or a
// fixed memory budget, code that runs inside CUDA stream capture (where a
// device allocation is not allowed), or a real-time loop that cannot afford
// the implicit synchronisation of an allocation.  For them this file offers
// the plane-contact detection of the solver as a stand-alone call on buffers
// the caller already owns.  Its only working memory is a file-scope
// `static __device__` array, so the call itself allocates nothing.
//
// The work is the rule of bvh_model.cpp:72-94 with the plane SDF of
// sdf_model.cpp:52-64 - every surface vertex with n.x + d < 0 becomes a
// contact at q = x + |n.x + d| n - written out in the order of the caller's
// surface list (a stable compaction: per-block hit counts, an exclusive scan
// of those counts, then a block-local ranked write).
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "../../include/sbs_gpu.h"

namespace {

constexpr uint32_t kNaBlock = 256;
constexpr uint32_t kNaMaxBlocks = 4096;
constexpr uint32_t kNaMaxSurface = kNaBlock * kNaMaxBlocks;  // 1,048,576 surface vertices

// Scratch: [0, kNaMaxBlocks) per-block hit counts, [kNaMaxBlocks, 2 kNaMaxBlocks)
// their exclusive scan.  32 KB, held by every device that loads the library
// until the process exits.  Every call rewrites the entries it reads, so no
// clearing is needed between calls; calls that overlap on the GPU race on it.
static __device__ __align__(256) uint32_t g_noalloc_scratch[2 * kNaMaxBlocks];

struct PlaneF {
    float nx, ny, nz, d;
};

__device__ __forceinline__ bool na_hit(const float* x, const uint32_t* surf, uint32_t n_surf, uint32_t n_verts,
                                       uint32_t i, const PlaneF& p, float* sd_out, uint32_t* v_out) {
    if (i >= n_surf) return false;
    const uint32_t v = surf[i];
    if (v >= n_verts) return false;  // never read outside the caller's position buffer
    const float px = x[3ull * v], py = x[3ull * v + 1], pz = x[3ull * v + 2];
    const float sd = p.nx * px + p.ny * py + p.nz * pz + p.d;
    *sd_out = sd;
    *v_out = v;
    return sd < 0.0f;
}

__global__ void k_na_count(const float* x, const uint32_t* surf, uint32_t n_surf, uint32_t n_verts, PlaneF p,
                           uint32_t* scratch) {
    const uint32_t i = blockIdx.x * kNaBlock + threadIdx.x;
    float sd;
    uint32_t v;
    const int hit = na_hit(x, surf, n_surf, n_verts, i, p, &sd, &v) ? 1 : 0;
    const int cnt = __syncthreads_count(hit);
    if (threadIdx.x == 0) scratch[blockIdx.x] = (uint32_t)cnt;
}

// One CTA of 1024 threads: exclusive scan of nblocks (<= 4096) counts.
__global__ void k_na_scan(uint32_t* scratch, uint32_t nblocks, uint32_t* count_out) {
    __shared__ uint32_t part[1024];
    const uint32_t t = threadIdx.x;
    uint32_t local[4], sum = 0;
    for (int k = 0; k < 4; ++k) {
        const uint32_t b = t * 4 + k;
        local[k] = b < nblocks ? scratch[b] : 0u;
        sum += local[k];
    }
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {  // Hillis-Steele inclusive scan
        const uint32_t add = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += add;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;  // exclusive prefix of this thread's group
    for (int k = 0; k < 4; ++k) {
        const uint32_t b = t * 4 + k;
        if (b < nblocks) scratch[kNaMaxBlocks + b] = run;
        run += local[k];
    }
    if (t == 1023) *count_out = part[1023];
}

__global__ void k_na_write(const float* x, const uint32_t* surf, uint32_t n_surf, uint32_t n_verts, PlaneF p,
                           const uint32_t* scratch, uint32_t* out_verts, float* out_q) {
    __shared__ uint32_t warp_base[kNaBlock / 32];
    const uint32_t i = blockIdx.x * kNaBlock + threadIdx.x;
    float sd = 0.0f;
    uint32_t v = 0;
    const bool hit = na_hit(x, surf, n_surf, n_verts, i, p, &sd, &v);
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t mask = __ballot_sync(0xffffffffu, hit);
    if (lane == 0) warp_base[wid] = __popc(mask);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t w = 0; w < kNaBlock / 32; ++w) {
            const uint32_t c = warp_base[w];
            warp_base[w] = run;
            run += c;
        }
    }
    __syncthreads();
    if (!hit) return;
    const uint32_t pos = scratch[kNaMaxBlocks + blockIdx.x] + warp_base[wid] + __popc(mask & ((1u << lane) - 1u));
    const float ad = fabsf(sd);
    out_verts[pos] = v;
    out_q[3ull * pos] = x[3ull * v] + p.nx * ad;
    out_q[3ull * pos + 1] = x[3ull * v + 1] + p.ny * ad;
    out_q[3ull * pos + 2] = x[3ull * v + 2] + p.nz * ad;
}

std::mutex g_na_mutex;
uint32_t* g_na_ptr[256] = {};

// Device address of the scratch array on the current device, looked up once
// per device (the name is only a host-side stand-in for it).  The cached
// address belongs to the device's context of that moment: after a
// cudaDeviceReset in the same process it is stale, so the entry point must
// not be used after one.
sbs_status na_scratch(uint32_t** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return SBS_ECUDA;
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_ptr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) return SBS_ECUDA;
        g_na_ptr[dev] = static_cast<uint32_t*>(p);
    }
    *out = g_na_ptr[dev];
    return SBS_OK;
}

}  // namespace

extern "C" sbs_status sbs_gpu_plane_contacts_noalloc(const float* x, uint32_t n_verts, const uint32_t* surface,
                                                     uint32_t n_surface, const double normal[3], double d,
                                                     uint32_t* contact_verts, float* contact_points,
                                                     uint32_t* count, void* stream) {
    if (!x || !surface || !normal || !contact_verts || !contact_points || !count) return SBS_EINVAL;
    if (n_surface > kNaMaxSurface) return SBS_EINVAL;  // more than 1,048,576 surface vertices
    const double l = sqrt(normal[0] * normal[0] + normal[1] * normal[1] + normal[2] * normal[2]);
    if (!(l > 0.0) || !(d == d)) return SBS_EINVAL;
    // An error left by earlier work on this thread is not this call's: report
    // it without clearing it and enqueue nothing.
    if (cudaPeekAtLastError() != cudaSuccess) return SBS_ECUDA;
    uint32_t* scratch = nullptr;
    sbs_status st = na_scratch(&scratch);
    if (st != SBS_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const PlaneF p{(float)(normal[0] / l), (float)(normal[1] / l), (float)(normal[2] / l), (float)(d / l)};
    const uint32_t nb = n_surface == 0 ? 1 : (n_surface + kNaBlock - 1) / kNaBlock;
    k_na_count<<<nb, kNaBlock, 0, s>>>(x, surface, n_surface, n_verts, p, scratch);
    if (cudaGetLastError() != cudaSuccess) return SBS_ECUDA;
    k_na_scan<<<1, 1024, 0, s>>>(scratch, nb, count);
    if (cudaGetLastError() != cudaSuccess) return SBS_ECUDA;
    k_na_write<<<nb, kNaBlock, 0, s>>>(x, surface, n_surface, n_verts, p, scratch, contact_verts, contact_points);
    return cudaGetLastError() == cudaSuccess ? SBS_OK : SBS_ECUDA;
}
