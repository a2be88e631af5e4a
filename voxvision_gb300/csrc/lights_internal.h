/*
 * lights_internal.h -- layouts of the light manager and its M-tree inside
 * libvoxtrees_cuda (lights.c), and the flat image the device searches.
 */
#ifndef VOX_LIGHTS_INTERNAL_H
#define VOX_LIGHTS_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#include "../../include/voxrnd.h"
#include "../../include/voxtrees.h"

#ifdef __cplusplus
extern "C" {
#endif

#define VOX_MTREE_MAX_CHILDREN 9          /* mtree.h:44 */

struct vox_mtree_node {                   /* mtree.h:46-56 */
    struct vox_sphere bounding_sphere;
    struct vox_mtree_node *parent;
    unsigned int leaf;
    unsigned int num;
    union {
        struct vox_mtree_node *children[VOX_MTREE_MAX_CHILDREN + 1];
        struct vox_sphere *spheres;       /* MAX + 1 spheres */
    } data;
};

struct vox_light_manager {                /* lights.c:11-14 */
    vox_dot ambient_light;
    struct vox_mtree_node *bound_lights;
    uint64_t version;                     /* bumped by every change: device copies follow it */
};

/* Flat copy of a light manager for the device.  Node record (8 floats):
 * bounding-sphere centre xyz, squared radius; then as u32 leaf flag, count,
 * first child record (inner) or first sphere record (leaf), 0.  The root is
 * record 0 and an inner node's children are consecutive records.  Sphere
 * record (8 floats): centre xyz, squared radius, colour rgb, radius. */
struct lights_image {
    float *nodes, *spheres;
    size_t n_nodes, n_spheres;
    unsigned depth;
    vox_dot ambient;
};

int lights_flatten(const struct vox_light_manager *lm, struct lights_image *img);
void lights_image_free(struct lights_image *img);

#ifdef __cplusplus
}
#endif

#endif
