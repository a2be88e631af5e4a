/* flatten.h -- host flattener of struct vox_node trees (see pool_layout.h). */
#ifndef VOX_FLATTEN_H
#define VOX_FLATTEN_H

#include <cstdint>
#include <vector>

#include "../../include/voxtrees.h"

struct uint4_host {
    uint32_t x, y, z, w;
};

struct FlatTree {
    std::vector<uint4_host> units;                     // the pool image
    std::vector<const vox_node *> preorder;            // pre-order id -> host node
    std::vector<uint32_t> rec_of_id;                   // pre-order id -> record offset
    uint64_t n_inner, n_leaf, n_dense, n_dots, depth;
    float voxel[3];
};

/* 0 on success, -1 when a leaf holds 2^30 voxels or more, -2 when the pool
 * would exceed VOXP_MAX_UNITS. */
int vox_flatten(const vox_node *root, const float voxel[3], FlatTree *out);

/* Walks the pool image from the root record and checks that every offset a
 * traversal can follow stays inside the pool and that every node is reached
 * exactly once; 0 when the image is sound. */
int vox_flatten_validate(const FlatTree &f);

#endif
