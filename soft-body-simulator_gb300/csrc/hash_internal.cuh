// Device layout of the spatial hash used for body-body contacts (hash_kernels.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "xpbd_internal.cuh"

namespace sbs {

struct HashDev {
    float inv_h;                  // 1 / cell size, rounded to float
    float depth;                  // contact depth limit (the cell size)
    int self;                     // 1: contacts within a body too
    uint32_t mask;                // table capacity - 1 (power of two, >= 2 x surface vertices)
    unsigned long long* keys;     // [cap] cell keys, ~0 = empty
    uint32_t* count;              // [cap] surface vertices per cell
    uint32_t* start;              // [cap] exclusive scan of count
    uint32_t* fill;               // [cap] fill cursor
    uint32_t* tile_sums;          // scan scratch: per 1024-slot tile
    uint32_t* tile_scan;
    uint32_t* tile_sums2;
    uint32_t* tile_scan2;
    uint32_t* vslot;              // [n_surf] table slot of each surface vertex
    uint32_t* entries;            // [n_surf] surface vertices grouped by cell
    uint32_t* vbody;              // [V] body id of each vertex
    uint8_t* bmask;               // [T] boundary faces of each tet slot (faces_copy order)
    uint32_t* query;              // [n_query] tet slots with at least one boundary face
    uint32_t n_query;
    unsigned long long* best;     // [V] (orderable d << 32) | ~slot, 0 = none
    float4* bc_q;                 // [V] contact point, w = 1 when the vertex has a body contact
    float4* bc_n;                 // [V] contact normal
    unsigned long long* cand;     // candidate pairs (vertex << 32 | slot), nullable
    unsigned long long cand_cap;
    unsigned long long* n_cand;   // candidate count of the last detection
};

cudaError_t launch_body_detect(const SceneDev& s, const HashDev& hd, cudaStream_t st);

}  // namespace sbs
