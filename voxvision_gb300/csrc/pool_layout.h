/*
 * pool_layout.h -- the device image of one voxtrees octree.
 *
 * The whole tree lives in one array of 16-byte units (uint4), so every load
 * the traversal makes is an aligned 16-byte vector load.  Every node is one
 * 3-unit record, so one round trip brings everything a node visit needs:
 *
 *   unit 0  {bmin.x, bmin.y, bmin.z, bmax.x}
 *   unit 1  {bmax.y, bmax.z, meta,   link  }
 *   unit 2  inner: {centre.x, centre.y, centre.z, 0}
 *           leaf : {pre-order id, voxel count, 0, 0}
 *           dense: {0, 0, 0, 0}
 *
 *   meta  bits 0-1  kind: 0 inner, 1 leaf (regular or overflowed), 2 dense
 *         inner: bits 8-15 child mask (bit o set = octant o non-NULL)
 *         leaf : bits 2-31 voxel count
 *   link  inner: unit offset of its child block, the records of its k
 *                non-NULL children in octant order (3k units);
 *         leaf : unit offset of its voxels, n units {x, y, z, 0} of voxel
 *                min-corners in the reference's order;
 *         dense: its pre-order id.
 *
 * The root record sits at unit 0.  Child blocks are laid out depth first,
 * so a subtree occupies one contiguous stretch of the pool.  Stack entries
 * carry unit offsets in 28 bits; the pool is therefore limited to 2^28
 * units (4 GiB) per tree.
 *
 * The algorithmic bytes of a search are counted independently of this
 * layout: 32 per node whose box is tested (box + kind/link), 16 more per
 * inner node entered (centre), 16 per voxel tested.
 */
#ifndef VOX_POOL_LAYOUT_H
#define VOX_POOL_LAYOUT_H

#include <stdint.h>

#define VOXP_KIND_INNER 0u
#define VOXP_KIND_LEAF  1u
#define VOXP_KIND_DENSE 2u

#define VOXP_REC_UNITS  3u

#define VOXP_OFF_BITS   28
#define VOXP_OFF_MASK   ((1u << VOXP_OFF_BITS) - 1u)
#define VOXP_MAX_UNITS  (1u << VOXP_OFF_BITS)

/* Root offset of an empty tree. */
#define VOXP_EMPTY      0xFFFFFFFFu

#endif
