// Layout of the cluster-resident execution mode (cluster_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "xpbd_internal.cuh"

namespace sbs {

constexpr int kClusterMaxBlock = 512;

// One group of whole bodies run by one thread-block cluster: vertices
// [v0, v0 + nv) in library order, colour table entries
// [col_base, col_base + n_col] of ClusterDev::col_start / col_split.
struct GroupDesc {
    uint32_t v0, nv, col_base, n_col, lb_base;
};

struct ClusterDev {
    GroupDesc* groups;
    uint32_t n_groups;
    // per group, colour-major then rank: n_col * C + 1 tet-slot offsets; the
    // tets of (colour c, rank r) are those of colour c owning most of their
    // vertices in rank r's slice
    uint32_t* col_start;
    uint32_t* lam_base;    // per group: n_col * C offsets into the CTA's multiplier array
    uint32_t lcap;         // multipliers per CTA (max tets owned by one CTA)
    uint4* tet_packed;     // per tet slot: vertex as (cluster rank << 24) | slice offset;
                           // bit 31 of .x set for a stable Neo-Hookean tet
    uint32_t stage;        // tet records per staging buffer (most tets one CTA has in one
                           // colour), 0: records are read from global memory in the phase
    uint8_t* vflags;       // per vertex: bit 0 = surface vertex
    uint32_t cluster_size;
    uint32_t slice;        // vertices per CTA slice
    uint32_t xn_minus_xi;  // byte offset from the xi slice to the xn slice
    int body;              // 1: body-body contacts (records below)
    const float4* bc_q;    // [V] body contact point, w != 0 when present
    const float4* bc_n;    // [V] body contact normal, w = slot in the global list (bits)
};

// Dynamic shared memory of one CTA for `slice` vertices, `planes` planes and
// an optional body-contact slot: two staging buffers of `stage` tet records
// (packed ids and the three DmInv rows, 64 bytes per tet), xi, xn, v, contact
// records and body normals (float4), global contact slots and the contact
// vertex list (uint32), the multipliers of the CTA's tets.
inline size_t cluster_smem_bytes(uint32_t slice, int planes, int body, uint32_t lcap, uint32_t stage = 0) {
    const size_t S = (size_t)planes + (body ? 1 : 0);
    return 2 * 64 * (size_t)stage + (size_t)slice * (3 * 16 + S * 16 + (body ? 16 : 0) + S * 4 + 4) +
           2 * sizeof(float) * (size_t)lcap;
}

cudaError_t cluster_configure(int block, size_t smem);
cudaError_t cluster_max_active(int cluster_size, int block, size_t smem, int* n);
cudaError_t launch_cluster_frame(const SceneDev& s, const ClusterDev& c, const StepParams& p, double t0,
                                 int n_clusters, int block, size_t smem, cudaStream_t st);
cudaError_t launch_store_time(double* t, double v, cudaStream_t st);

}  // namespace sbs
