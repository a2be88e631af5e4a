/*
 * lights.c -- the reference's light manager (src/voxrnd/lights.c) and the
 * M-tree of light spheres it keeps (src/voxtrees/mtree.c), on the host.
 *
 * The shadowless lights are spheres in an M-tree; a lit pixel adds, in the
 * tree's traversal order, the contribution of every sphere that contains the
 * hit point.  The float sums depend on that order, so the tree is built by
 * the reference's own insertion steps (choice of the nearest child, node
 * split at the two farthest centres, bounding-sphere updates propagated to
 * the root) and removal steps, with the same float operations; the device
 * copy (lights_flatten) keeps the children's order.  Compiled with
 * -ffp-contract=off like the rest of the host code, so each operation rounds
 * as in the reference's scalar build.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "lights_internal.h"

#define EXPORT __attribute__((visibility("default")))

/* geom.c:133-139 vox_sqr_metric, scalar build (powf(d, 2) is d * d). */
static float sqr_metric(const float *a, const float *b)
{
    float r = 0.0f;
    for (int i = 0; i < 3; i++) {
        float d = a[i] - b[i];
        r += d * d;
    }
    return r;
}

static int same_dot(const float *a, const float *b) { return memcmp(a, b, sizeof(vox_dot)) == 0; }

static struct vox_mtree_node *node_new(int leaf)
{
    struct vox_mtree_node *n = calloc(1, sizeof *n);
    if (!n) return NULL;
    n->leaf = (unsigned)leaf;
    if (leaf) {
        n->data.spheres = calloc(VOX_MTREE_MAX_CHILDREN + 1, sizeof(struct vox_sphere));
        if (!n->data.spheres) { free(n); return NULL; }
    }
    return n;
}

static const struct vox_sphere *item(const struct vox_mtree_node *n, unsigned i)
{
    return n->leaf ? &n->data.spheres[i] : &n->data.children[i]->bounding_sphere;
}

/* mtree.c:21-56: grow bounding sphere `bs` to hold sphere `s`, with the
 * smallest radius; returns 1 if it changed. */
static int grow_sphere(const struct vox_sphere *s, struct vox_sphere *bs)
{
    float dist = sqrtf(sqr_metric(s->center, bs->center));
    float crit = (1 + (bs->radius - s->radius) / dist) / 2;
    if (crit < 0) {
        *bs = *s;
        return 1;
    }
    if (crit < 1) {
        bs->radius = (s->radius + bs->radius + dist) / 2;
        bs->sqr_radius = (float)pow(bs->radius, 2);
        for (int i = 0; i < 3; i++) {
            float d = bs->center[i] - s->center[i];   /* vox_dot_sub, scmul, add */
            d = crit * d;
            bs->center[i] = s->center[i] + d;
        }
        return 1;
    }
    return 0;
}

/* mtree.c:58-74 */
static int node_sphere(struct vox_mtree_node *n)
{
    int changed = 0;
    n->bounding_sphere = *item(n, 0);
    for (unsigned i = 1; i < n->num; i++) changed += grow_sphere(item(n, i), &n->bounding_sphere);
    return changed != 0;
}

/* mtree.c:76-87 */
static void propagate(struct vox_mtree_node *n)
{
    while (n && node_sphere(n)) n = n->parent;
}

/* mtree.c:89-112: centres of the two items farthest apart (first pair found
 * at the largest distance).  All centres equal: the first item's, twice. */
static void farthest(const struct vox_mtree_node *n, float *c1, float *c2)
{
    float maxd = 0.0f;
    memcpy(c1, item(n, 0)->center, sizeof(vox_dot));
    memcpy(c2, item(n, 0)->center, sizeof(vox_dot));
    for (unsigned i = 0; i < n->num; i++) {
        for (unsigned j = i + 1; j < n->num; j++) {
            float d = sqr_metric(item(n, i)->center, item(n, j)->center);
            if (d > maxd) {
                memcpy(c1, item(n, i)->center, sizeof(vox_dot));
                memcpy(c2, item(n, j)->center, sizeof(vox_dot));
                maxd = d;
            }
        }
    }
}

/* mtree.c:114-180: split a node holding MAX+1 items in two around the
 * farthest centres; returns the last node not changed by the split (beyond
 * its bounding sphere) or the new root.  NULL if memory runs out. */
static struct vox_mtree_node *split(struct vox_mtree_node *n)
{
    struct vox_mtree_node *parent = n->parent, *res = parent;
    struct vox_mtree_node *a = node_new((int)n->leaf), *b = node_new((int)n->leaf);
    if (!a || !b) return NULL;
    a->parent = b->parent = parent;
    vox_dot c1, c2;
    farthest(n, c1, c2);
    for (unsigned i = 0; i < n->num; i++) {
        float d1 = sqr_metric(item(n, i)->center, c1);
        float d2 = sqr_metric(item(n, i)->center, c2);
        struct vox_mtree_node *to = d1 < d2 ? a : b;
        if (n->leaf) {
            to->data.spheres[to->num] = n->data.spheres[i];
        } else {
            to->data.children[to->num] = n->data.children[i];
            n->data.children[i]->parent = to;
        }
        to->num++;
    }
    node_sphere(a);
    node_sphere(b);
    if (n->leaf) free(n->data.spheres);
    if (parent) {
        for (unsigned i = 0; i < parent->num; i++)
            if (parent->data.children[i] == n) parent->data.children[i] = a;
        parent->data.children[parent->num++] = b;
        free(n);
        propagate(parent);
        if (parent->num == VOX_MTREE_MAX_CHILDREN + 1) res = split(parent);
    } else {
        free(n);
        res = node_new(0);
        if (!res) return NULL;
        res->num = 2;
        res->data.children[0] = a;
        res->data.children[1] = b;
        node_sphere(res);
        a->parent = b->parent = res;
    }
    return res;
}

/* mtree.c:182-216 */
EXPORT struct vox_mtree_node *vox_mtree_contains_sphere(const struct vox_mtree_node *n, const struct vox_sphere *s)
{
    if (!n) return NULL;
    if (!(sqr_metric(s->center, n->bounding_sphere.center) < n->bounding_sphere.sqr_radius)) return NULL;
    if (n->leaf) {
        for (unsigned i = 0; i < n->num; i++)
            if (same_dot(n->data.spheres[i].center, s->center) && n->data.spheres[i].radius == s->radius)
                return (struct vox_mtree_node *)n;
        return NULL;
    }
    for (unsigned i = 0; i < n->num; i++) {
        struct vox_mtree_node *r = vox_mtree_contains_sphere(n->data.children[i], s);
        if (r) return r;
    }
    return NULL;
}

/* mtree.c:218-253: descend to the child whose bounding-sphere centre is
 * nearest (first of equals), append to the leaf, split if full. */
static struct vox_mtree_node *add_helper(struct vox_mtree_node *n, const struct vox_sphere *s, int *oom)
{
    float sqr_radius = (float)pow(s->radius, 2);
    if (!n) {
        struct vox_mtree_node *r = node_new(1);
        if (!r) { *oom = 1; return NULL; }
        r->bounding_sphere = *s;
        r->bounding_sphere.sqr_radius = sqr_radius;
        r->num = 1;
        r->data.spheres[0] = *s;
        r->data.spheres[0].sqr_radius = sqr_radius;
        return r;
    }
    if (n->leaf) {
        n->data.spheres[n->num] = *s;
        n->data.spheres[n->num].sqr_radius = sqr_radius;
        n->num++;
        propagate(n);
        if (n->num == VOX_MTREE_MAX_CHILDREN + 1) {
            struct vox_mtree_node *r = split(n);
            if (!r) *oom = 1;
            return r;
        }
        return n;
    }
    struct vox_mtree_node *child = n->data.children[0];
    float mind = INFINITY;
    for (unsigned i = 0; i < n->num; i++) {
        float d = sqr_metric(s->center, n->data.children[i]->bounding_sphere.center);
        if (d < mind) {
            mind = d;
            child = n->data.children[i];
        }
    }
    return add_helper(child, s, oom);
}

/* mtree.c:255-267 */
EXPORT int vox_mtree_add_sphere(struct vox_mtree_node **root, const struct vox_sphere *s)
{
    if (!(s->radius > 0) || vox_mtree_contains_sphere(*root, s)) return 0;
    int oom = 0;
    struct vox_mtree_node *n = add_helper(*root, s, &oom);
    if (oom || !n) return 0;
    if (n->parent == NULL) *root = n;
    return 1;
}

/* mtree.c:269-322: delete a leaf; a parent left with one child is replaced
 * by that child.  Returns the last node modified (NULL: the tree is empty). */
static struct vox_mtree_node *delete_leaf(struct vox_mtree_node *n)
{
    struct vox_mtree_node *parent = n->parent;
    vox_mtree_destroy(n);
    if (!parent) return NULL;
    unsigned i = 0;
    while (i < parent->num && parent->data.children[i] != n) i++;
    if (parent->num == 2) {
        struct vox_mtree_node *other = parent->data.children[1 - i], *top = parent->parent;
        free(parent);
        other->parent = top;
        if (!top) return other;
        unsigned k = 0;
        while (k < top->num && top->data.children[k] != parent) k++;
        top->data.children[k] = other;
        propagate(top);
        return top;
    }
    parent->num--;
    memmove(&parent->data.children[i], &parent->data.children[i + 1],
            sizeof(struct vox_mtree_node *) * (parent->num - i));
    parent->data.children[parent->num] = NULL;
    propagate(parent);
    return parent;
}

/* mtree.c:324-368 */
EXPORT int vox_mtree_remove_sphere(struct vox_mtree_node **root, const struct vox_sphere *s)
{
    struct vox_mtree_node *leaf = vox_mtree_contains_sphere(*root, s);
    if (!(s->radius > 0) || !leaf) return 0;
    struct vox_mtree_node *last = leaf;
    if (leaf->num == 1) {
        last = delete_leaf(leaf);
    } else {
        unsigned i = 0;
        while (i < leaf->num &&
               !(same_dot(leaf->data.spheres[i].center, s->center) && leaf->data.spheres[i].radius == s->radius))
            i++;
        memmove(&leaf->data.spheres[i], &leaf->data.spheres[i + 1],
                sizeof(struct vox_sphere) * (leaf->num - i - 1));
        leaf->num--;
        propagate(leaf);
    }
    if (last == NULL || last->parent == NULL) *root = last;
    return 1;
}

EXPORT void vox_mtree_destroy(struct vox_mtree_node *n)
{
    if (!n) return;
    if (n->leaf) {
        free(n->data.spheres);
    } else {
        for (unsigned i = 0; i < n->num; i++) vox_mtree_destroy(n->data.children[i]);
    }
    free(n);
}

/* mtree.c:384-416: the M-tree printed node by node, depth first (the text
 * the reference prints, for the same debugging use). */
EXPORT void vox_mtree_dump(const struct vox_mtree_node *node)
{
    printf("Node %p ", (const void *)node);
    if (!node) {
        printf("empty node\n");
        return;
    }
    printf("%s, parent=%p\n", node->leaf ? "leaf" : "inner node", (void *)node->parent);
    printf("Bounding sphere: <%7.4f, %7.4f, %7.4f>, %7.4f\n", node->bounding_sphere.center[0],
           node->bounding_sphere.center[1], node->bounding_sphere.center[2], node->bounding_sphere.radius);
    if (node->leaf) {
        printf("Leaf content (%u spheres):\n", node->num);
        for (unsigned i = 0; i < node->num; i++)
            printf("<%7.4f, %7.4f, %7.4f>, %7.4f\n", node->data.spheres[i].center[0],
                   node->data.spheres[i].center[1], node->data.spheres[i].center[2],
                   node->data.spheres[i].radius);
        printf("==========\n");
    } else {
        printf("Node children\n");
        for (unsigned i = 0; i < node->num; i++) printf("%p ", (void *)node->data.children[i]);
        printf("\n==========\n");
        for (unsigned i = 0; i < node->num; i++) vox_mtree_dump(node->data.children[i]);
    }
}

EXPORT unsigned int vox_mtree_items(const struct vox_mtree_node *n)
{
    if (!n) return 0;
    if (n->leaf) return n->num;
    unsigned c = 0;
    for (unsigned i = 0; i < n->num; i++) c += vox_mtree_items(n->data.children[i]);
    return c;
}

/* mtree.c:463-493: every sphere containing `dot`, depth first, children in
 * order; a one-sphere leaf inside whose bounding sphere the dot lies yields
 * its sphere without a second test. */
EXPORT void vox_mtree_spheres_containing_f(const struct vox_mtree_node *n, const vox_dot dot,
                                    void (*callback)(const struct vox_sphere *s, void *arg), void *arg)
{
    if (!n || !(sqr_metric(n->bounding_sphere.center, dot) < n->bounding_sphere.sqr_radius)) return;
    if (n->leaf) {
        if (n->num == 1) {
            callback(&n->data.spheres[0], arg);
            return;
        }
        for (unsigned i = 0; i < n->num; i++)
            if (sqr_metric(n->data.spheres[i].center, dot) < n->data.spheres[i].sqr_radius)
                callback(&n->data.spheres[i], arg);
        return;
    }
    for (unsigned i = 0; i < n->num; i++) vox_mtree_spheres_containing_f(n->data.children[i], dot, callback, arg);
}

/* ------------------------------------------------------------------------
 * The light manager (lights.c:1-116)
 * ---------------------------------------------------------------------- */

static int valid_colour(const float *c)
{
    for (int i = 0; i < 3; i++)
        if (c[i] < 0 || c[i] > 1) return 0;
    return 1;
}

EXPORT struct vox_light_manager *vox_make_light_manager(void)
{
    struct vox_light_manager *lm = calloc(1, sizeof *lm);
    if (!lm) return NULL;
    lm->ambient_light[0] = lm->ambient_light[1] = lm->ambient_light[2] = 1.0f;
    return lm;
}

EXPORT void vox_destroy_light_manager(struct vox_light_manager *lm)
{
    if (!lm) return;
    vox_mtree_destroy(lm->bound_lights);
    free(lm);
}

EXPORT int vox_set_ambient_light(struct vox_light_manager *lm, const vox_dot color)
{
    if (!valid_colour(color)) return 0;
    memcpy(lm->ambient_light, color, sizeof(vox_dot));
    lm->version++;
    return 1;
}

EXPORT int vox_insert_shadowless_light(struct vox_light_manager *lm, const vox_dot center, float radius,
                                const vox_dot color)
{
    if (!valid_colour(color)) return 0;
    struct vox_sphere s;
    memset(&s, 0, sizeof s);
    memcpy(s.center, center, sizeof(vox_dot));
    memcpy(s.color, color, sizeof(vox_dot));
    s.radius = radius;
    int ok = vox_mtree_add_sphere(&lm->bound_lights, &s);
    if (ok) lm->version++;
    return ok;
}

EXPORT int vox_delete_shadowless_light(struct vox_light_manager *lm, const vox_dot center, float radius)
{
    struct vox_sphere s;
    memset(&s, 0, sizeof s);
    memcpy(s.center, center, sizeof(vox_dot));
    s.radius = radius;
    int ok = vox_mtree_remove_sphere(&lm->bound_lights, &s);
    if (ok) lm->version++;
    return ok;
}

EXPORT void vox_delete_shadowless_lights(struct vox_light_manager *lm)
{
    vox_mtree_destroy(lm->bound_lights);
    lm->bound_lights = NULL;
    lm->version++;
}

EXPORT int vox_shadowless_lights_number(const struct vox_light_manager *lm)
{
    return (int)vox_mtree_items(lm->bound_lights);
}

/* ------------------------------------------------------------------------
 * Device image of a light manager
 * ---------------------------------------------------------------------- */

static void count(const struct vox_mtree_node *n, size_t *nodes, size_t *spheres, unsigned depth, unsigned *maxd)
{
    if (!n) return;
    (*nodes)++;
    if (depth > *maxd) *maxd = depth;
    if (n->leaf) {
        *spheres += n->num;
        return;
    }
    for (unsigned i = 0; i < n->num; i++) count(n->data.children[i], nodes, spheres, depth + 1, maxd);
}

/* Writes the records of n's children (n's record is at `self`), depth first:
 * an inner node's children occupy consecutive records, a leaf's spheres
 * consecutive sphere records, both in the tree's order. */
static void place(const struct vox_mtree_node *n, size_t self, struct lights_image *img, size_t *next_node,
                  size_t *next_sphere)
{
    float *rec = img->nodes + 8 * self;
    uint32_t *meta = (uint32_t *)(rec + 4);
    memcpy(rec, n->bounding_sphere.center, sizeof(vox_dot));
    rec[3] = n->bounding_sphere.sqr_radius;
    meta[0] = n->leaf;
    meta[1] = n->num;
    meta[3] = 0;
    if (n->leaf) {
        meta[2] = (uint32_t)*next_sphere;
        for (unsigned i = 0; i < n->num; i++) {
            const struct vox_sphere *s = &n->data.spheres[i];
            float *sp = img->spheres + 8 * (*next_sphere)++;
            memcpy(sp, s->center, sizeof(vox_dot));
            sp[3] = s->sqr_radius;
            memcpy(sp + 4, s->color, sizeof(vox_dot));
            sp[7] = s->radius;
        }
        return;
    }
    size_t first = *next_node;
    meta[2] = (uint32_t)first;
    *next_node += n->num;
    for (unsigned i = 0; i < n->num; i++) place(n->data.children[i], first + i, img, next_node, next_sphere);
}

int lights_flatten(const struct vox_light_manager *lm, struct lights_image *img)
{
    memset(img, 0, sizeof *img);
    memcpy(img->ambient, lm->ambient_light, sizeof(vox_dot));
    size_t nodes = 0, spheres = 0;
    unsigned maxd = 0;
    count(lm->bound_lights, &nodes, &spheres, 1, &maxd);
    img->n_nodes = nodes;
    img->n_spheres = spheres;
    img->depth = maxd;
    if (nodes == 0) return 0;
    img->nodes = calloc(nodes * 8, sizeof(float));
    img->spheres = calloc((spheres ? spheres : 1) * 8, sizeof(float));
    if (!img->nodes || !img->spheres) {
        lights_image_free(img);
        return -1;
    }
    size_t next_node = 1, next_sphere = 0;
    place(lm->bound_lights, 0, img, &next_node, &next_sphere);
    return 0;
}

void lights_image_free(struct lights_image *img)
{
    free(img->nodes);
    free(img->spheres);
    img->nodes = img->spheres = NULL;
}
