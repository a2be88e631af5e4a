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
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/voxtrees.h"

#define EXPORT __attribute__((visibility("default")))

static void destroy_nodes(struct vox_node *tree);

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

EXPORT struct vox_node *vox_make_tree_host(vox_dot set[], size_t n)
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
    destroy_nodes(root);
    return NULL;
}

static void destroy_nodes(struct vox_node *tree)
{
    if (!tree) return;
    if (tree->flags & VOX_LEAF) {
        free(tree->data.dots);
    } else if (!(tree->flags & VOX_LEAF_MASK)) {
        for (int i = 0; i < 8; i++) destroy_nodes(tree->data.inner.children[i]);
    }
    free(tree);
}

/* Drops cached device copies of trees that contain `node` (dropin_search.cpp). */
void vox_dropin_forget_containing(const struct vox_node *node);

EXPORT void vox_destroy_tree(struct vox_node *tree)
{
    if (!tree) return;
    // a later tree may be allocated at the same addresses: no device copy of
    // this one may outlive it
    vox_dropin_forget_containing(tree);
    destroy_nodes(tree);
}

EXPORT size_t vox_voxels_in_tree(const struct vox_node *tree)
{
    return tree ? tree->dots_num : 0;
}

/* geom.c:125-147: distances summed axis by axis from 0, in axis order. */
EXPORT float vox_abs_metric(const vox_dot dot1, const vox_dot dot2)
{
    float r = 0;
    for (int i = 0; i < 3; i++) r += fabsf(dot1[i] - dot2[i]);
    return r;
}

EXPORT float vox_sqr_metric(const vox_dot dot1, const vox_dot dot2)
{
    float r = 0;
    for (int i = 0; i < 3; i++) {
        float d = dot1[i] - dot2[i];
        r += d * d;
    }
    return r;
}

EXPORT float vox_sqr_norm(const vox_dot dot)
{
    float r = 0;
    for (int i = 0; i < 3; i++) r += dot[i] * dot[i];
    return r;
}

/* geom.c:44-51: octant of `dot` around `center`, bit i set when center[i] > dot[i]. */
EXPORT int get_subspace_idx(const vox_dot center, const vox_dot dot)
{
    int r = 0;
    for (int i = 0; i < 3; i++) r |= (center[i] > dot[i]) << i;
    return r;
}

/* tree.c:868-918: the tree printed node by node, depth first (the text the
 * reference prints, for the same debugging use). */
EXPORT void vox_dump_tree(const struct vox_node *tree)
{
    if (!tree) return;
    const int inner = !(tree->flags & VOX_LEAF_MASK);
    printf("Node %p %s\n", (const void *)tree,
           (tree->flags & VOX_LEAF) ? "LEAF" : (tree->flags & VOX_DENSE_LEAF) ? "DENSE LEAF" : "INNER");
    printf("Bounding box min <%f, %f, %f>\n", tree->bounding_box.min[0], tree->bounding_box.min[1],
           tree->bounding_box.min[2]);
    printf("Bounding box max <%f, %f, %f>\n", tree->bounding_box.max[0], tree->bounding_box.max[1],
           tree->bounding_box.max[2]);
    printf("Number of voxels %u\n", tree->dots_num);
    if (tree->flags & VOX_LEAF) {
        printf("Dots:\n");
        for (unsigned i = 0; i < tree->dots_num; i++)
            printf("<%f, %f, %f>\n", tree->data.dots[i][0], tree->data.dots[i][1], tree->data.dots[i][2]);
    } else if (inner) {
        printf("Center <%f, %f, %f>\n", tree->data.inner.center[0], tree->data.inner.center[1],
               tree->data.inner.center[2]);
        printf("Children:\n");
        for (int i = 0; i < 8; i++) printf("%p\n", (void *)tree->data.inner.children[i]);
    }
    printf("------Node ends here------\n");
    if (inner) {
        for (int i = 0; i < 8; i++) vox_dump_tree(tree->data.inner.children[i]);
        printf("=======Node and children end here=======\n");
    }
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

/* ------------------------------------------------------------------------
 * Tree editing (tree.c:425-866): insertion and deletion of single voxels,
 * restated step for step.  The shape of the edited tree -- which leaves
 * become dense, where a dense leaf is split, which inner nodes disappear --
 * decides every later search, so each case follows the reference.  Bounding
 * boxes grow on insertion and are not shrunk on deletion, as there.
 * ---------------------------------------------------------------------- */


/* tree.c:185-194 */
static void align_to_grid(vox_dot d)
{
    for (int i = 0; i < 3; i++) {
        float t = floorf(d[i] / vox_voxel[i]);
        d[i] = vox_voxel[i] * t;
    }
}

/* tree.c:197-209: widen a box to hold the voxel at d. */
static void grow_box(struct vox_box *b, const vox_dot d)
{
    vox_dot top;
    for (int i = 0; i < 3; i++) top[i] = d[i] + vox_voxel[i];
    for (int i = 0; i < 3; i++) {
        b->min[i] = (d[i] < b->min[i]) ? d[i] : b->min[i];
        b->max[i] = (top[i] > b->max[i]) ? top[i] : b->max[i];
    }
}

/* geom.c:5-11 voxel_in_box: half-open box. */
static int voxel_inside(const struct vox_box *b, const vox_dot d)
{
    for (int i = 0; i < 3; i++)
        if (d[i] < b->min[i] || d[i] >= b->max[i]) return 0;
    return 1;
}

/* geom.c:44-51 get_subspace_idx (no direction correction). */
static int subspace(const float *c, const float *d)
{
    return (c[0] > d[0]) | ((c[1] > d[1]) << 1) | ((c[2] > d[2]) << 2);
}

/* geom.c:192-196 get_dimensions */
static void box_dims(const struct vox_box *b, size_t dim[3])
{
    for (int i = 0; i < 3; i++) dim[i] = (size_t)((b->max[i] - b->min[i]) / vox_voxel[i]);
}

static int same_voxel(const float *a, const float *b) { return memcmp(a, b, sizeof(vox_dot)) == 0; }

/* tree.c:377-423 flatten_tree: the voxels of a subtree, dense leaves walked
 * x, then y, then z with the coordinate advanced by one voxel each step. */
static size_t collect(const struct vox_node *t, vox_dot *out)
{
    if (!t) return 0;
    if (t->flags & VOX_LEAF) {
        memcpy(out, t->data.dots, t->dots_num * sizeof(vox_dot));
        return t->dots_num;
    }
    if (t->flags & VOX_DENSE_LEAF) {
        size_t dim[3], n = 0;
        vox_dot cur;
        box_dims(&t->bounding_box, dim);
        cur[0] = t->bounding_box.min[0];
        for (size_t i = 0; i < dim[0]; i++) {
            cur[1] = t->bounding_box.min[1];
            for (size_t j = 0; j < dim[1]; j++) {
                cur[2] = t->bounding_box.min[2];
                for (size_t k = 0; k < dim[2]; k++) {
                    memcpy(out[n++], cur, sizeof(vox_dot));
                    cur[2] += vox_voxel[2];
                }
                cur[1] += vox_voxel[1];
            }
            cur[0] += vox_voxel[0];
        }
        return n;
    }
    size_t n = 0;
    for (int i = 0; i < 8; i++) n += collect(t->data.inner.children[i], out + n);
    return n;
}

/* tree.c:425-436 */
EXPORT struct vox_node *vox_rebuild_tree(const struct vox_node *tree)
{
    if (!tree) return NULL;
    vox_dot *set = malloc((tree->dots_num ? tree->dots_num : 1) * sizeof(vox_dot));
    if (!set) return NULL;
    collect(tree, set);
    struct vox_node *t = vox_make_tree(set, tree->dots_num);
    free(set);
    return t;
}

/* tree.c:438-458 voxel_in_tree */
static int holds_voxel(const struct vox_node *t, const vox_dot d)
{
    while (t && voxel_inside(&t->bounding_box, d)) {
        if (t->flags & VOX_DENSE_LEAF) return 1;
        if (t->flags & VOX_LEAF) {
            for (unsigned i = 0; i < t->dots_num; i++)
                if (same_voxel(d, t->data.dots[i])) return 1;
            return 0;
        }
        t = t->data.inner.children[subspace(t->data.inner.center, d)];
    }
    return 0;
}

static struct vox_node *inner_node(const struct vox_box *box, unsigned dots, const vox_dot centre)
{
    struct vox_node *n = malloc(sizeof(struct vox_node));
    if (!n) return NULL;
    n->bounding_box = *box;
    n->flags = 0;
    n->dots_num = dots;
    memcpy(n->data.inner.center, centre, sizeof(vox_dot));
    memset(n->data.inner.children, 0, sizeof n->data.inner.children);
    return n;
}

/* geom.c:33-42 closest_vertex */
static void nearest_corner(const struct vox_box *b, const vox_dot d, vox_dot res)
{
    for (int i = 0; i < 3; i++) {
        float d1 = fabsf(b->min[i] - d[i]);
        float d2 = fabsf(b->max[i] - d[i]);
        res[i] = (d1 < d2) ? b->min[i] : b->max[i];
    }
}

/* geom.c:169-182 divide_box: the octant idx of box around centre (bit i set:
 * the lower half along i); 0 if it is empty. */
static int octant_box(const struct vox_box *b, const vox_dot c, struct vox_box *res, int idx)
{
    *res = *b;
    for (int i = 0; i < 3; i++) {
        if (idx & (1 << i)) res->max[i] = c[i];
        else res->min[i] = c[i];
        if (res->min[i] == res->max[i]) return 0;
    }
    return 1;
}

static int insert_at(struct vox_node **slot, const vox_dot d);

/* tree.c:461-502 insert_in_big_dense: the dense leaf and the new voxel
 * become two children of a new inner node split at the leaf's box corner
 * nearest to the voxel. */
static struct vox_node *insert_beside_dense(struct vox_node *t, const vox_dot d)
{
    vox_dot centre, mid;
    nearest_corner(&t->bounding_box, d, centre);
    struct vox_box box = t->bounding_box;
    grow_box(&box, d);
    struct vox_node *n = inner_node(&box, t->dots_num + 1, centre);
    if (!n) return NULL;
    for (int i = 0; i < 3; i++) mid[i] = (t->bounding_box.min[i] + t->bounding_box.max[i]) / 2;
    int i1 = subspace(centre, mid), i2 = subspace(centre, d);
    n->data.inner.children[i1] = t;
    if (insert_at(&n->data.inner.children[i2], d)) {
        free(n);
        return NULL;
    }
    return n;
}

/* tree.c:505-608 vox_insert_voxel_: the voxel is known not to be in the
 * tree.  Returns nonzero if memory ran out. */
static int insert_at(struct vox_node **slot, const vox_dot d)
{
    for (;;) {
        struct vox_node *t = *slot, *node = t;
        if (!t) {
            vox_dot one[1];
            memcpy(one[0], d, sizeof(vox_dot));
            node = vox_make_tree_host(one, 1);
            if (!node) return 1;
            *slot = node;
            return 0;
        }
        struct vox_box before = t->bounding_box;
        grow_box(&t->bounding_box, d);
        if (box_is_full(&t->bounding_box, (size_t)t->dots_num + 1)) {
            if (t->flags & VOX_DENSE_LEAF) {
                t->dots_num++;
            } else {
                node = vox_make_dense_leaf(&t->bounding_box);
                if (!node) return 1;
                destroy_nodes(t);
            }
            *slot = node;
            return 0;
        }
        if (t->flags & VOX_DENSE_LEAF) {
            t->bounding_box = before;
            if (t->dots_num < VOX_MAX_DOTS) {
                /* a small dense leaf becomes an ordinary leaf */
                vox_dot set[VOX_MAX_DOTS];
                collect(t, set);
                memcpy(set[t->dots_num], d, sizeof(vox_dot));
                node = vox_make_tree_host(set, t->dots_num + 1);
                if (!node) return 1;
                destroy_nodes(t);
            } else {
                node = insert_beside_dense(t, d);
                if (!node) return 1;
            }
            *slot = node;
            return 0;
        }
        if (t->flags & VOX_LEAF) {
            if (t->dots_num < VOX_MAX_DOTS) {
                memcpy(t->data.dots[t->dots_num], d, sizeof(vox_dot));
                t->dots_num++;
                return 0;
            }
            /* a full leaf becomes a subtree; an overflowed leaf (only built
             * from duplicate voxels, which the reference cannot extend
             * either) is rebuilt with the new voxel */
            vox_dot *set = malloc(((size_t)t->dots_num + 1) * sizeof(vox_dot));
            if (!set) return 1;
            memcpy(set, t->data.dots, t->dots_num * sizeof(vox_dot));
            memcpy(set[t->dots_num], d, sizeof(vox_dot));
            node = vox_make_tree_host(set, t->dots_num + 1);
            free(set);
            if (!node) return 1;
            destroy_nodes(t);
            *slot = node;
            return 0;
        }
        /* inner node: count the voxel and go down */
        t->dots_num++;
        slot = &t->data.inner.children[subspace(t->data.inner.center, d)];
    }
}

/* tree.c:610-619: 1 if inserted, 0 if the voxel was already there (the
 * voxel is first snapped to the grid, in place). */
EXPORT int vox_insert_voxel(struct vox_node **tree, vox_dot voxel)
{
    align_to_grid(voxel);
    if (holds_voxel(*tree, voxel)) return 0;
    if (*tree) vox_dropin_forget_containing(*tree);
    return insert_at(tree, voxel) ? 0 : 1;
}

EXPORT int vox_insert_voxel_coord(struct vox_node **tree, float x, float y, float z)
{
    vox_dot d = {x, y, z};
    return vox_insert_voxel(tree, d);
}

/* tree.c:634-691 delete_from_dense_stripe: deletion from a dense leaf one
 * voxel thick in two directions; NULL if the leaf is not such a stripe. */
static struct vox_node *delete_from_stripe(struct vox_node *t, const vox_dot d)
{
    size_t dim[3];
    int ones = 0, axis = 0;
    box_dims(&t->bounding_box, dim);
    for (int i = 0; i < 3; i++) {
        if (dim[i] == 1) ones++;
        else axis = i;
    }
    if (ones != 2) return NULL;
    if (same_voxel(t->bounding_box.min, d)) {            /* first voxel of the stripe */
        t->dots_num--;
        t->bounding_box.min[axis] += vox_voxel[axis];
        return t;
    }
    vox_dot past;
    for (int i = 0; i < 3; i++) past[i] = d[i] + vox_voxel[i];
    if (same_voxel(t->bounding_box.max, past)) {         /* last voxel */
        t->dots_num--;
        t->bounding_box.max[axis] -= vox_voxel[axis];
        return t;
    }
    /* a voxel inside: two dense halves under one inner node */
    struct vox_node *n = inner_node(&t->bounding_box, t->dots_num - 1, d);
    if (!n) return NULL;
    struct vox_box b;
    octant_box(&t->bounding_box, d, &b, 1 << axis);
    n->data.inner.children[1 << axis] = vox_make_dense_leaf(&b);
    octant_box(&t->bounding_box, d, &b, 0);
    struct vox_node *c = vox_make_dense_leaf(&b);
    n->data.inner.children[0] = c;
    c->dots_num--;
    c->bounding_box.min[axis] += vox_voxel[axis];
    destroy_nodes(t);
    return n;
}

/* tree.c:693-752 delete_from_big_dense */
static struct vox_node *delete_from_dense(struct vox_node *t, const vox_dot d)
{
    struct vox_node *n = delete_from_stripe(t, d);
    if (n) return n;
    struct vox_box b;
    if (same_voxel(t->bounding_box.min, d)) {
        /* the corner voxel: the dense boxes around the voxel past it */
        vox_dot past;
        for (int i = 0; i < 3; i++) past[i] = d[i] + vox_voxel[i];
        n = inner_node(&t->bounding_box, t->dots_num - 1, past);
        if (!n) return NULL;
        for (int i = 0; i < 7; i++)
            if (octant_box(&t->bounding_box, past, &b, i)) n->data.inner.children[i] = vox_make_dense_leaf(&b);
        destroy_nodes(t);
        return n;
    }
    n = inner_node(&t->bounding_box, t->dots_num - 1, d);
    if (!n) return NULL;
    for (int i = 0; i < 8; i++)
        if (octant_box(&t->bounding_box, d, &b, i)) n->data.inner.children[i] = vox_make_dense_leaf(&b);
    /* the voxel is now the corner of octant 0 */
    n->data.inner.children[0] = delete_from_dense(n->data.inner.children[0], d);
    destroy_nodes(t);
    return n;
}

/* tree.c:754-842 vox_delete_voxel_: the voxel is known to be in the tree. */
static void delete_at(struct vox_node **slot, const vox_dot d)
{
    for (;;) {
        struct vox_node *t = *slot;
        if (t->dots_num == 1) {
            destroy_nodes(t);
            *slot = NULL;
            return;
        }
        if (t->flags & VOX_LEAF) {
            unsigned i = 0;
            while (i < t->dots_num && !same_voxel(t->data.dots[i], d)) i++;
            t->dots_num--;
            memmove(t->data.dots + i, t->data.dots + i + 1, sizeof(vox_dot) * (t->dots_num - i));
            return;
        }
        if (t->flags & VOX_DENSE_LEAF) {
            if (t->dots_num <= VOX_MAX_DOTS) {
                struct vox_node *n = delete_from_stripe(t, d);
                if (n) {
                    *slot = n;
                    return;
                }
                vox_dot set[VOX_MAX_DOTS];
                collect(t, set);
                unsigned i = 0;
                while (i < t->dots_num && !same_voxel(set[i], d)) i++;
                memmove(set + i, set + i + 1, sizeof(vox_dot) * (t->dots_num - i - 1));
                *slot = vox_make_tree_host(set, t->dots_num - 1);
                destroy_nodes(t);
            } else {
                *slot = delete_from_dense(t, d);
            }
            return;
        }
        struct vox_node *child = t->data.inner.children[subspace(t->data.inner.center, d)];
        if (child->dots_num == t->dots_num) {
            /* the only child: it takes its parent's place */
            *slot = child;
            free(t);
            continue;
        }
        t->dots_num--;
        slot = &t->data.inner.children[subspace(t->data.inner.center, d)];
    }
}

/* tree.c:844-853: 1 if deleted, 0 if the voxel was not there (snapped to the
 * grid first, in place). */
EXPORT int vox_delete_voxel(struct vox_node **tree, vox_dot voxel)
{
    align_to_grid(voxel);
    if (!holds_voxel(*tree, voxel)) return 0;
    vox_dropin_forget_containing(*tree);
    delete_at(tree, voxel);
    return 1;
}

EXPORT int vox_delete_voxel_coord(struct vox_node **tree, float x, float y, float z)
{
    vox_dot d = {x, y, z};
    return vox_delete_voxel(tree, d);
}
