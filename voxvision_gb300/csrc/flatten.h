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

/* The node layout of a voxvision built with SSE_INTRIN (its default on x86):
 * vox_dot is float[4] aligned to 16 bytes, so struct vox_box takes 32 bytes
 * and struct vox_node 128, its union starting at byte 48
 * (voxvision.h.in:45-57, tree.h:22-38).  Same member names as vox_node. */
typedef float vox_dot16[4] __attribute__((aligned(16)));
struct vox_box16 {
    vox_dot16 min, max;
};
struct vox_node16 {
    vox_box16 bounding_box;
    unsigned int flags;
    unsigned int dots_num;
    union {
        vox_dot16 *dots;
        struct {
            vox_dot16 center;
            vox_node16 *children[8];
        } inner;
    } data;
};
static_assert(sizeof(vox_node16) == 128, "SSE-layout node is 128 bytes");

/* 0 on success, -1 when a leaf holds 2^30 voxels or more, -2 when the pool
 * would exceed VOXP_MAX_UNITS.  vox_flatten16 reads an SSE-layout tree and
 * produces the same image a scalar-layout tree of the same nodes gives; its
 * pre-order table holds the vox_node16 pointers (as opaque vox_node
 * pointers). */
int vox_flatten(const vox_node *root, const float voxel[3], FlatTree *out);
int vox_flatten16(const vox_node16 *root, const float voxel[3], FlatTree *out);

/* Walks the pool image from the root record and checks that every offset a
 * traversal can follow stays inside the pool and that every node is reached
 * exactly once; 0 when the image is sound. */
int vox_flatten_validate(const FlatTree &f);

#endif
