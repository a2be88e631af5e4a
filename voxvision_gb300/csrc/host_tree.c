/*
 * host_tree.c -- host-side octree construction of the voxtrees API.
 *
 * The tree the GPU searches must be the reference's tree node for node and
 * dot for dot: the search order, the leaf loop's tie-breaking and every
 * reported leaf depend on it.  So construction follows src/voxtrees/tree.c
 * (scalar branch) step for step -- bounding box :138-155, density test
 * geom.c:157-167, subdivision centre :125-136, the in-place swapping
 * partition :166-183 and the recursion with its overflow leaf :249-338 --
 * written here as an explicit work list instead of recursion.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/voxtrees.h"

#define EXPORT __attribute__((visibility("default")))

EXPORT vox_dot vox_voxel = {1.0f, 1.0f, 1.0f};

EXPORT void vox_set_voxel_size(float x, float y, float z)
{
    vox_voxel[0] = x;
    vox_voxel[1] = y;
    vox_voxel[2] = z;
}

/* Smallest box holding every voxel of the set (min corners, max corner plus
 * one voxel). */
static void set_box(const vox_dot *set, size_t n, struct vox_box *box)
{
    float lo[3] = {set[0][0], set[0][1], set[0][2]};
    float hi[3] = {set[0][0], set[0][1], set[0][2]};
    for (size_t i = 0; i < n; i++) {
        for (int a = 0; a < 3; a++) {
            float v = set[i][a];
            if (v < lo[a]) lo[a] = v;
            else if (v > hi[a]) hi[a] = v;
        }
    }
    for (int a = 0; a < 3; a++) {
        box->min[a] = lo[a];
        box->max[a] = hi[a] + vox_voxel[a];
    }
}

/* True when n voxels fill the box completely (a "dense" set). */
static int box_is_full(const struct vox_box *box, size_t n)
{
    float ext0 = box->max[0] - box->min[0];
    float ext1 = box->max[1] - box->min[1];
    float ext2 = box->max[2] - box->min[2];
    float box_volume = ext0 * ext1 * ext2;
    float voxel_volume = vox_voxel[0] * vox_voxel[1] * vox_voxel[2];
    return fabsf((float)n * voxel_volume - box_volume) < voxel_volume;
}

/* Mean of the voxels relative to the box corner, snapped up to the grid. */
static void split_point(const vox_dot *set, size_t n, const struct vox_box *box, float *c)
{
    float acc[3] = {0.0f, 0.0f, 0.0f};
    for (size_t i = 0; i < n; i++)
        for (int a = 0; a < 3; a++)
            acc[a] = (set[i][a] - box->min[a]) + acc[a];
    for (int a = 0; a < 3; a++) {
        float mean = acc[a] / (float)n + box->min[a];
        c[a] = ceilf(mean / vox_voxel[a]) * vox_voxel[a];
    }
}

static inline int octant(const float *c, const float *p)
{
    return (c[0] > p[0]) | ((c[1] > p[1]) << 1) | ((c[2] > p[2]) << 2);
}

/* Move the voxels of octant `oct` found in [from, n) to the front of that
 * range, swapping each one with the first not-yet-claimed slot. */
static size_t claim_octant(vox_dot *set, size_t n, size_t from, int oct, const float *c)
{
    size_t next = from;
    for (size_t i = from; i < n; i++) {
        if (octant(c, set[i]) != oct) continue;
        float t0 = set[next][0], t1 = set[next][1], t2 = set[next][2];
        set[next][0] = set[i][0]; set[next][1] = set[i][1]; set[next][2] = set[i][2];
        set[i][0] = t0; set[i][1] = t1; set[i][2] = t2;
        next++;
    }
    return next;
}

static struct vox_node *new_leaf(const vox_dot *set, size_t n, size_t capacity, unsigned flags)
{
    struct vox_node *node = malloc(sizeof(struct vox_node));
    if (!node) return NULL;
    node->flags = flags;
    node->dots_num = (unsigned)n;
    node->data.dots = malloc(capacity * sizeof(vox_dot));
    if (!node->data.dots) { free(node); return NULL; }
    memcpy(node->data.dots, set, n * sizeof(vox_dot));
    return node;
}

typedef struct {
    vox_dot *set;
    size_t n;
    struct vox_node **slot;   /* where the built node is stored */
} build_job;

EXPORT struct vox_node *vox_make_tree(vox_dot set[], size_t n)
{
    struct vox_node *root = NULL;
    if (n == 0) return NULL;

    size_t cap = 64, top = 0;
    build_job *jobs = malloc(cap * sizeof(build_job));
    if (!jobs) return NULL;
    jobs[top++] = (build_job){set, n, &root};

    while (top) {
        build_job job = jobs[--top];
        struct vox_box box;
        set_box(job.set, job.n, &box);
        struct vox_node *node;

        if (box_is_full(&box, job.n)) {
            node = malloc(sizeof(struct vox_node));
            if (!node) goto oom;
            node->flags = VOX_DENSE_LEAF;
            node->dots_num = (unsigned)job.n;
        } else if (job.n <= VOX_MAX_DOTS) {
            node = new_leaf(job.set, job.n, VOX_MAX_DOTS, VOX_LEAF);
            if (!node) goto oom;
        } else {
            float c[3];
            split_point(job.set, job.n, &box, c);
            /* Partition octant by octant; an octant that takes the whole set at
             * the start means no split is possible: one overflowed leaf. */
            size_t bounds[9];
            int overflow = 0;
            bounds[0] = 0;
            for (int o = 0; o < 8; o++) {
                bounds[o + 1] = claim_octant(job.set, job.n, bounds[o], o, c);
                if (bounds[o] == 0 && bounds[o + 1] == job.n) { overflow = 1; break; }
            }
            if (overflow) {
                node = new_leaf(job.set, job.n, job.n, VOX_LEAF | VOX_OVERFLOW);
                if (!node) goto oom;
            } else {
                node = malloc(sizeof(struct vox_node));
                if (!node) goto oom;
                node->flags = 0;
                node->dots_num = (unsigned)job.n;
                node->data.inner.center[0] = c[0];
                node->data.inner.center[1] = c[1];
                node->data.inner.center[2] = c[2];
                if (top + 8 > cap) {
                    cap *= 2;
                    build_job *grown = realloc(jobs, cap * sizeof(build_job));
                    if (!grown) { free(node); goto oom; }
                    jobs = grown;
                }
                for (int o = 7; o >= 0; o--) {
                    size_t cnt = bounds[o + 1] - bounds[o];
                    node->data.inner.children[o] = NULL;
                    if (cnt)
                        jobs[top++] = (build_job){job.set + bounds[o], cnt,
                                                  &node->data.inner.children[o]};
                }
            }
        }
        node->bounding_box = box;
        *job.slot = node;
    }
    free(jobs);
    return root;

oom:
    free(jobs);
    vox_destroy_tree(root);
    return NULL;
}

EXPORT void vox_destroy_tree(struct vox_node *tree)
{
    if (!tree) return;
    if (tree->flags & VOX_LEAF) {
        free(tree->data.dots);
    } else if (!(tree->flags & VOX_LEAF_MASK)) {
        for (int i = 0; i < 8; i++) vox_destroy_tree(tree->data.inner.children[i]);
    }
    free(tree);
}

EXPORT size_t vox_voxels_in_tree(const struct vox_node *tree)
{
    return tree ? tree->dots_num : 0;
}

EXPORT void vox_bounding_box(const struct vox_node *tree, struct vox_box *box)
{
    *box = tree->bounding_box;
}

EXPORT struct vox_node *vox_make_dense_leaf(const struct vox_box *box)
{
    struct vox_node *node = malloc(sizeof(struct vox_node));
    if (!node) return NULL;
    node->bounding_box = *box;
    node->flags = VOX_DENSE_LEAF;
    size_t d0 = (size_t)((box->max[0] - box->min[0]) / vox_voxel[0]);
    size_t d1 = (size_t)((box->max[1] - box->min[1]) / vox_voxel[1]);
    size_t d2 = (size_t)((box->max[2] - box->min[2]) / vox_voxel[2]);
    node->dots_num = (unsigned)(d0 * d1 * d2);
    return node;
}
