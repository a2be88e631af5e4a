/*
 * voxtrees.h -- the voxtrees part of the reference API, as libvoxtrees_cuda
 * exports it (drop-in for src/voxtrees/tree.h and src/voxtrees/search.h of
 * shamazmazum/voxvision, scalar build).
 *
 * The node layout is the reference's own (tree.h:13-38 with the scalar
 * vox_dot of voxvision.h.in:57) so that trees built by either library can be
 * handed to vox_cuda_tree_upload.  Tree construction stays on the host and
 * follows tree.c:249-338 step for step; the searches run on the GPU.
 */
#ifndef VOXTREES_GB300_H
#define VOXTREES_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef float vox_dot[3];     /* voxvision.h.in:57 (SSE_INTRIN off) */
typedef float vox_quat[4];    /* voxvision.h.in:58 */

struct vox_box {              /* voxvision.h.in:79-83 */
    vox_dot min;
    vox_dot max;
};

#define VOX_LEAF 1            /* tree.h:15-18 */
#define VOX_DENSE_LEAF 2
#define VOX_LEAF_MASK 3
#define VOX_OVERFLOW 4
#define VOX_MAX_DOTS 7        /* params.h:29 */

typedef struct {              /* tree.h:22-26 */
    vox_dot center;
    struct vox_node *children[8];
} vox_inner_data;

struct vox_node {             /* tree.h:28-38 */
    struct vox_box bounding_box;
    unsigned int flags;
    unsigned int dots_num;
    union {
        vox_dot *dots;
        vox_inner_data inner;
    } data;
};

/* Voxel size (tree.c:11).  Read by vox_make_tree and by vox_cuda_tree_upload. */
extern vox_dot vox_voxel;

/* tree.h:60 -- build a tree; `set` is reordered in place and may be freed after.
 * Large sets are built on the GPU when one is present (the same tree, and the
 * same order of `set`; see vox_cuda_make_tree_gpu_min in voxtrees_cuda.h). */
struct vox_node *vox_make_tree(vox_dot set[], size_t n);
/* Extension: vox_make_tree on the host only (tree.c:249-338). */
struct vox_node *vox_make_tree_host(vox_dot set[], size_t n);
/* tree.h:67 */
void vox_destroy_tree(struct vox_node *tree);
/* tree.h:72 */
size_t vox_voxels_in_tree(const struct vox_node *tree);
/* datareader.h:40-53 -- `filename` as given, else in the data directory the
 * library was built with (VOX_DATA_PATH, if any), else in $VOXVISION_DATA
 * ($HOME/.voxvision when unset); the path found goes to `fullpath` (PATH_MAX
 * bytes).  1 if found. */
int vox_find_data_file(const char *filename, char *fullpath);
/* tree.h:130 -- print the tree to stdout, node by node (the reference's text). */
void vox_dump_tree(const struct vox_node *tree);
/* geom.h:59-73 -- L1 distance, squared distance, squared norm (summed in axis order). */
float vox_abs_metric(const vox_dot dot1, const vox_dot dot2);
float vox_sqr_metric(const vox_dot dot1, const vox_dot dot2);
float vox_sqr_norm(const vox_dot dot);
/* geom.h:87 -- octant of `dot` around `center` (bit i: center[i] > dot[i]). */
int get_subspace_idx(const vox_dot center, const vox_dot dot);
/* tree.h:77 */
void vox_bounding_box(const struct vox_node *tree, struct vox_box *box);
/* tree.h:140 */
struct vox_node *vox_make_dense_leaf(const struct vox_box *box);
/* tree.h:149 */
void vox_set_voxel_size(float x, float y, float z);

/* tree.h:88-122 -- editing.  The voxel is first snapped to the voxel grid
 * in place; insertion returns 1 if the voxel was added (0: already there),
 * deletion 1 if it was removed (0: not there).  *tree may change (a new root,
 * or NULL when the last voxel goes).  Cached device copies of the edited
 * tree (the single-query calls below) are dropped; a vox_cuda_tree of it
 * must be refreshed with vox_cuda_tree_refresh. */
int vox_insert_voxel(struct vox_node **tree, vox_dot voxel);
int vox_insert_voxel_coord(struct vox_node **tree, float x, float y, float z);
int vox_delete_voxel(struct vox_node **tree, vox_dot voxel);
int vox_delete_voxel_coord(struct vox_node **tree, float x, float y, float z);
/* tree.h:86 -- a new tree built by vox_make_tree from the voxels of `tree`. */
struct vox_node *vox_rebuild_tree(const struct vox_node *tree);

/* search.h:24-26 -- one ray, run on the GPU.  The tree (or the tree that
 * contains `tree`, which may be any of its nodes) is uploaded on first use and
 * kept until it is edited through this library or vox_cuda_forget_tree is
 * called; after editing a tree with other code, call that before the next
 * search.  Returns the leaf the reference returns, or NULL; `res` is
 * written on a hit only. */
const struct vox_node *vox_ray_tree_intersection(const struct vox_node *tree, const vox_dot origin,
                                                 const vox_dot dir, vox_dot res);
/* search.h:36-37 -- one ball query, run on the GPU (same caching). */
int vox_tree_ball_collidep(const struct vox_node *tree, const vox_dot center, float radius);

/* Drop the cached device copy of the tree rooted at `root` (no-op if none). */
void vox_cuda_forget_tree(const struct vox_node *root);

/* ---- M-trees of spheres (mtree.h:17-146): the light manager keeps its
 * lights in one.  Same layout, same insertion, split and removal steps (the
 * order in which a search visits spheres follows from them).  The block
 * variant vox_mtree_spheres_containing needs clang blocks and is not
 * provided; vox_mtree_spheres_containing_f is. */
struct vox_sphere {           /* mtree.h:17-40 */
    vox_dot center;
    vox_dot color;
    float radius;
    float sqr_radius;         /* set by the library */
};

struct vox_mtree_node;

/* mtree.h:73 -- 1 if added (radius > 0 and no sphere with the same centre
 * and radius in the tree), 0 otherwise; *root may change. */
int vox_mtree_add_sphere(struct vox_mtree_node **root, const struct vox_sphere *s);
/* mtree.h:86 -- 1 if a sphere with the same centre and radius was removed. */
int vox_mtree_remove_sphere(struct vox_mtree_node **root, const struct vox_sphere *s);
/* mtree.h:91 */
void vox_mtree_destroy(struct vox_mtree_node *root);
/* mtree.h:104 -- the leaf holding a sphere with the same centre and radius, or NULL. */
struct vox_mtree_node *vox_mtree_contains_sphere(const struct vox_mtree_node *root, const struct vox_sphere *s);
/* mtree.h:110 -- number of spheres. */
unsigned int vox_mtree_items(const struct vox_mtree_node *root);
/* mtree.h:98 -- print the M-tree to stdout, node by node (the reference's text). */
void vox_mtree_dump(const struct vox_mtree_node *root);
/* mtree.h:138-140 -- call callback(s, arg) for every sphere containing dot. */
void vox_mtree_spheres_containing_f(const struct vox_mtree_node *root, const vox_dot dot,
                                    void (*callback)(const struct vox_sphere *s, void *arg), void *arg);

#ifdef __cplusplus
}
#endif
#endif
