/*
 * oracle.h -- CPU restatement of the voxtrees ray/ball search path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA
 * product is compared against.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py load it; the product library never links or
 * calls it.
 *
 * Every function restates the reference algorithm (shamazmazum/voxvision,
 * scalar build, SSE_INTRIN off) in plain C, compiled with -ffp-contract=off
 * so that each float operation rounds separately, exactly as in the
 * reference's own build with contraction off.  The restatement itself is
 * pinned against the reference's sources compiled unmodified (oracle/_ref)
 * through the golden vectors under tests/golden/.
 */
#ifndef VOX_ORACLE_H
#define VOX_ORACLE_H

#include <stddef.h>
#include <stdint.h>

/* Node layout of the reference, scalar vox_dot (src/voxtrees/tree.h:22-38,
 * src/voxvision.h.in:79-83).  The layout must match byte for byte because
 * the same host trees are handed to the CUDA uploader. */
typedef float orc_dot[3];

struct orc_box { orc_dot min, max; };

typedef struct {
    orc_dot center;
    struct orc_node *children[8];
} orc_inner;

struct orc_node {
    struct orc_box bounding_box;
    unsigned int flags;
    unsigned int dots_num;
    union {
        orc_dot *dots;
        orc_inner inner;
    } data;
};

#define ORC_LEAF       1   /* tree.h:15 */
#define ORC_DENSE_LEAF 2   /* tree.h:16 */
#define ORC_LEAF_MASK  3   /* tree.h:17 */
#define ORC_OVERFLOW   4   /* tree.h:18 */
#define ORC_MAX_DOTS   7   /* params.h:29 */

/* Per-query work counters; they define the algorithmic bytes of a query. */
typedef struct {
    uint64_t nodes;   /* non-NULL nodes whose bounding box was tested */
    uint64_t inner;   /* inner nodes entered (their centre was read)   */
    uint64_t voxels;  /* leaf voxels tested                            */
} orc_counts;

/* Camera state consumed by screen2world (simple-camera.c:10-17,
 * doom-camera.c:8-15). kind 0 = simple-camera, 1 = doom-camera, 2 = any
 * other class, known by what its screen2world returns: pixel (x, y)'s
 * direction is rays[3 * (y * rays_w + x) ...]. */
typedef struct {
    int32_t kind;
    float position[3];
    float rotation[4];
    float mul, xsub, ysub;
    float sinphi, cosphi, k;
    const float *rays;
    int32_t rays_w;
} orc_camera;

void orc_set_voxel(float x, float y, float z);
void orc_get_voxel(float out[3]);

struct orc_node *orc_make_tree(float *set, size_t n);
void orc_destroy_tree(struct orc_node *tree);

const struct orc_node *orc_ray(const struct orc_node *tree, const float *origin,
                               const float *dir, float *res, int *slot,
                               orc_counts *cnt);
int orc_ball(const struct orc_node *tree, const float *center, float radius,
             orc_counts *cnt);

/* Pre-order numbering of the non-NULL nodes (node, then children 0..7). */
size_t orc_count_nodes(const struct orc_node *tree);
size_t orc_preorder(const struct orc_node *tree, const struct orc_node **out);

/* Batched, multi-threaded drivers.  leaf_id is the pre-order index of the
 * returned leaf (UINT32_MAX on a miss), slot the winning dot (0xFF for a
 * dense leaf or a miss); points are written only on a hit.  `root` may be any
 * node of the tree whose pre-order numbering is taken from `tree`. */
int orc_ray_batch(const struct orc_node *tree, const struct orc_node *root,
                  size_t n, const float *origins, const float *dirs,
                  uint32_t *leaf_id, uint8_t *slot, float *points,
                  uint64_t *counts3, int nthreads);
int orc_ball_batch(const struct orc_node *tree, size_t n, const float *centers,
                   const float *radii, uint8_t *hit, uint64_t *counts3,
                   int nthreads);

/* Per-ray work counters (nodes, inner, voxels), for cost distributions. */
int orc_ray_counts_per_ray(const struct orc_node *root, size_t n, const float *origins,
                           const float *dirs, uint32_t *per_ray, int nthreads);

void orc_screen2world(const orc_camera *cam, int sx, int sy, float *ray);

/* A simple-camera of field of view `fov` (horizontal when w > h) for a w x h
 * window at `position`, looking at `target`: the fields that
 * set_property_number("fov"), set_window_size, set_property_dot("position")
 * and look_at leave in the reference's camera (simple-camera.c:106-170). */
void orc_camera_simple(orc_camera *cam, const float position[3], const float target[3], int w, int h, float fov);

/* vox_render, quality BEST (renderer.c:200-319, branch :308) into a linear
 * ARGB8888 framebuffer; misses stay 0 (vox_redraw clears, renderer.c:324). */
int orc_render_best(const struct orc_node *tree, const orc_camera *cam,
                    int w, int h, const uint8_t *texture, uint32_t *argb,
                    uint64_t *counts3, int nthreads);

/* vox_render in any quality (renderer.c:215-318): BEST, FAST, ADAPTIVE,
 * ADAPTIVE with ray merging.  Pixels the reference leaves undrawn are 0. */
int orc_render_quality(const struct orc_node *tree, const orc_camera *cam,
                       int w, int h, unsigned quality, const uint8_t *texture,
                       uint32_t *argb, uint64_t *counts3, int nthreads);

/* Light manager (lights.c) with its M-tree (mtree.c), and frames of any
 * quality coloured with it (renderer.c:27-52).  The M-tree code of the
 * reference needs clang blocks and cannot be compiled here, so this
 * restatement is checked against the reference's own M-tree test
 * properties (orc_lights_verify, tests/tests.c:779-900) and against the
 * product's independent restatement through the GPU tests. */
typedef struct orc_lights orc_lights;
orc_lights *orc_lights_new(void);
void orc_lights_free(orc_lights *l);
int orc_lights_ambient(orc_lights *l, const float *color);
int orc_lights_insert(orc_lights *l, const float *center, float radius, const float *color);
int orc_lights_delete(orc_lights *l, const float *center, float radius);
int orc_lights_count(const orc_lights *l);
/* vox_get_light: writes the light at p; returns how many spheres contain p. */
int orc_lights_get(const orc_lights *l, const float *p, float *light);
/* 0 when the reference's M-tree invariants hold. */
int orc_lights_verify(const orc_lights *l);
int orc_render_lit(const struct orc_node *tree, const orc_camera *cam, int w, int h, unsigned quality,
                   const uint8_t *texture, const orc_lights *lights, uint32_t *argb, int nthreads);

/* Pre-order dump of a tree: per node flags, dots_num, box (6 floats), centre
 * (3 floats, inner nodes), child mask (inner nodes) and an offset into the
 * dots array (leaves).  Returns the node count; arrays must be sized by
 * orc_count_nodes() and the total number of stored dots. */
size_t orc_dump(const struct orc_node *tree, uint32_t *flags, uint32_t *dots_num,
                float *boxes, float *centers, uint8_t *child_mask,
                uint64_t *dot_offset, float *dots);
size_t orc_count_stored_dots(const struct orc_node *tree);
/* Rebuild a tree from such a dump (used for trees the reference built by
 * insertion, which the restated builder does not produce). */
struct orc_node *orc_from_dump(size_t nnodes, const uint32_t *flags,
                               const uint32_t *dots_num, const float *boxes,
                               const float *centers, const uint8_t *child_mask,
                               const uint64_t *dot_offset, const float *dots);

#endif
