/*
 * pool_layout.h -- the device image of one voxtrees octree.
 *
 * The whole tree lives in one array of 16-byte units (uint4), so every load
 * the traversal makes is an aligned 16-byte vector load:
 *
 *   node record  2 units   {bmin.x, bmin.y, bmin.z, bmax.x}
 *                          {bmax.y, bmax.z, meta,   link  }
 *   inner block  1 + 2k    {centre.x, centre.y, centre.z, 0} followed by the
 *                          records of the k non-NULL children in octant order
 *   leaf block   1 + n     {pre-order id, n, 0, 0} followed by n voxel
 *                          min-corners {x, y, z, 0}
 *
 *   meta  bits 0-1  kind: 0 inner, 1 leaf (regular or overflowed), 2 dense
 *         inner: bits 8-15 child mask (bit o set = octant o non-NULL)
 *         leaf : bits 2-31 voxel count
 *   link  inner: unit offset of its block;  leaf: unit offset of its first
 *         voxel (header one unit before);   dense: its pre-order id
 *
 * The root record sits at unit 0.  Blocks are laid out depth first, so a
 * subtree occupies one contiguous stretch of the pool.  Traversal stacks
 * carry unit offsets in 28 bits; the pool is therefore limited to 2^28 units
 * (4 GiB) per tree.
 *
 * Per node visit the traversal reads 32 bytes (the record), per inner node
 * entered 16 more (the centre), per voxel tested 16.
 */
#ifndef VOX_POOL_LAYOUT_H
#define VOX_POOL_LAYOUT_H

#include <stdint.h>

#define VOXP_KIND_INNER 0u
#define VOXP_KIND_LEAF  1u
#define VOXP_KIND_DENSE 2u

#define VOXP_OFF_BITS   28
#define VOXP_OFF_MASK   ((1u << VOXP_OFF_BITS) - 1u)
#define VOXP_MAX_UNITS  (1u << VOXP_OFF_BITS)

/* Root offset of an empty tree. */
#define VOXP_EMPTY      0xFFFFFFFFu

#endif
