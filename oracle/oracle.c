/*
 * oracle.c -- CPU restatement of the voxtrees ray/ball search path and of the
 * BEST-quality render loop.  TEST INFRASTRUCTURE ONLY (see oracle.h): the
 * product never links this file.
 *
 * Reference files restated here (paths within shamazmazum/voxvision):
 *   src/voxtrees/tree.c      vox_make_tree and its scalar helpers
 *   src/voxtrees/geom.c      hit_box, hit_plane_within_box, metrics, ...
 *   src/voxtrees/search.c    vox_ray_tree_intersection, vox_tree_ball_collidep
 *   src/voxrnd/renderer.c    vox_render (every quality), get_color
 *   src/voxrnd/lights.c      the light manager; src/voxtrees/mtree.c its M-tree
 *   src/voxrnd/simple-camera.c, doom-camera.c, vect-ops.c   screen2world
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

static float orc_voxel[3] = {1.0f, 1.0f, 1.0f};   /* tree.c:11 vox_voxel */

void orc_set_voxel(float x, float y, float z)
{
    orc_voxel[0] = x; orc_voxel[1] = y; orc_voxel[2] = z;
}

void orc_get_voxel(float out[3])
{
    out[0] = orc_voxel[0]; out[1] = orc_voxel[1]; out[2] = orc_voxel[2];
}

/* ------------------------------------------------------------------ */
/* geometry (geom.c, scalar branch)                                    */
/* ------------------------------------------------------------------ */

/* geom.c:13-31 fit_into_box: clamp, report whether the dot was inside. */
static int fit_into_box(const struct orc_box *box, const float *dot, float *res)
{
    int same = 1;
    for (int i = 0; i < 3; i++) {
        if (dot[i] < box->min[i]) { res[i] = box->min[i]; same = 0; }
        else if (dot[i] > box->max[i]) { res[i] = box->max[i]; same = 0; }
        else res[i] = dot[i];
    }
    return same;
}

/* geom.c:44-51 */
static int subspace_idx(const float *center, const float *dot)
{
    int r = 0;
    for (int i = 0; i < 3; i++) r |= (center[i] > dot[i]) << i;
    return r;
}

/* geom.c:53-65 */
static int corrected_subspace_idx(const float *center, const float *dot, const float *dir)
{
    int r = 0;
    for (int i = 0; i < 3; i++) {
        int a = (center[i] == dot[i]) ? (dir[i] < 0) : (center[i] > dot[i]);
        r |= a << i;
    }
    return r;
}

/* geom.c:69-99 hit_box: entry point of a ray into a closed box. */
static int hit_box(const struct orc_box *box, const float *origin, const float *dir, float *res)
{
    if (fit_into_box(box, origin, res)) return 1;
    int plane = 0;
    float maxd = -1;
    for (int i = 0; i < 3; i++) {
        float t = (res[i] - origin[i]) / dir[i];
        if (t > maxd) { plane = i; maxd = t; }
    }
    if (maxd <= 0) return 0;
    for (int i = 0; i < 3; i++) {
        if (i == plane) continue;
        float t = origin[i] + maxd * dir[i];
        if (t < box->min[i] || t > box->max[i]) return 0;
        res[i] = t;
    }
    return 1;
}

/* geom.c:101-123 hit_plane_within_box */
static int hit_plane_within_box(const float *origin, const float *dir, const float *planedot,
                                int p, float *res, const struct orc_box *box)
{
    float k = planedot[p] - origin[p];
    if (k == 0 || ((dir[p] < 0) != (k < 0))) return 0;
    k = k / dir[p];
    for (int i = 0; i < 3; i++) {
        res[i] = origin[i] + k * dir[i];
        if (res[i] < box->min[i] || res[i] > box->max[i]) return 0;
    }
    return 1;
}

/* geom.c:125-131: ((0 + |dx|) + |dy|) + |dz| */
static float abs_metric(const float *a, const float *b)
{
    float r = 0;
    for (int i = 0; i < 3; i++) r += fabsf(a[i] - b[i]);
    return r;
}

/* geom.c:133-139 (powf(d, 2.0) is d*d) */
static float sqr_metric(const float *a, const float *b)
{
    float r = 0;
    for (int i = 0; i < 3; i++) { float d = a[i] - b[i]; r += d * d; }
    return r;
}

/* geom.c:149-154 */
static int box_ball_interp(const struct orc_box *box, const float *center, float radius)
{
    float f[3];
    fit_into_box(box, center, f);
    return sqr_metric(f, center) < radius * radius;
}

/* geom.c:157-167 */
static int dense_set_p(const struct orc_box *box, size_t n)
{
    float size[3];
    for (int i = 0; i < 3; i++) size[i] = box->max[i] - box->min[i];
    float bbv = size[0] * size[1] * size[2];
    float vv = orc_voxel[0] * orc_voxel[1] * orc_voxel[2];
    return fabsf((float)n * vv - bbv) < vv;
}

/* ------------------------------------------------------------------ */
/* tree build (tree.c:125-338, scalar branch)                          */
/* ------------------------------------------------------------------ */

/* tree.c:138-155 */
static void calc_bounding_box(orc_dot *set, size_t n, struct orc_box *box)
{
    memcpy(box->min, set[0], sizeof(orc_dot));
    memcpy(box->max, set[0], sizeof(orc_dot));
    for (size_t i = 0; i < n; i++)
        for (int j = 0; j < 3; j++) {
            if (set[i][j] < box->min[j]) box->min[j] = set[i][j];
            else if (set[i][j] > box->max[j]) box->max[j] = set[i][j];
        }
    for (int j = 0; j < 3; j++) box->max[j] = box->max[j] + orc_voxel[j];
}

/* tree.c:125-136: mean of (dot - box.min), then aligned up to the voxel grid */
static void find_center(orc_dot *set, size_t n, const struct orc_box *box, float *res)
{
    res[0] = res[1] = res[2] = 0;
    for (size_t i = 0; i < n; i++)
        for (int j = 0; j < 3; j++) {
            float t = set[i][j] - box->min[j];
            res[j] = t + res[j];
        }
    for (int j = 0; j < 3; j++)
        res[j] = ceilf((res[j] / (float)n + box->min[j]) / orc_voxel[j]) * orc_voxel[j];
}

/* tree.c:166-183: stable-for-the-chosen, swapping partition */
static size_t sort_set(orc_dot *set, size_t n, size_t offset, int sub, const float *center)
{
    size_t counter = offset;
    for (size_t i = offset; i < n; i++) {
        if (subspace_idx(center, set[i]) == sub) {
            orc_dot tmp;
            memcpy(tmp, set[counter], sizeof(orc_dot));
            memcpy(set[counter], set[i], sizeof(orc_dot));
            memcpy(set[i], tmp, sizeof(orc_dot));
            counter++;
        }
    }
    return counter;
}

static struct orc_node *make_tree(orc_dot *set, size_t n)
{
    if (n == 0) return NULL;
    struct orc_node *node = calloc(1, sizeof(struct orc_node));
    struct orc_box box;
    calc_bounding_box(set, n, &box);
    int densep = dense_set_p(&box, n);
    int leafp = n <= ORC_MAX_DOTS;
    node->dots_num = (unsigned)n;
    node->bounding_box = box;
    if (densep) {
        node->flags = ORC_DENSE_LEAF;
    } else if (leafp) {
        node->data.dots = malloc(ORC_MAX_DOTS * sizeof(orc_dot));
        memcpy(node->data.dots, set, n * sizeof(orc_dot));
        node->flags = ORC_LEAF;
    } else {
        orc_inner *inner = &node->data.inner;
        size_t offset = 0;
        node->flags = 0;
        find_center(set, n, &node->bounding_box, inner->center);
        for (int idx = 0; idx < 8; idx++) {
            size_t noff = sort_set(set, n, offset, idx, inner->center);
            if (offset == 0 && noff == n) {
                /* tree.c:281-305: unsplittable set -> one overflowed leaf */
                node->flags = ORC_LEAF | ORC_OVERFLOW;
                node->data.dots = malloc(n * sizeof(orc_dot));
                memcpy(node->data.dots, set, n * sizeof(orc_dot));
                break;
            }
            inner->children[idx] = make_tree(set + offset, noff - offset);
            offset = noff;
        }
    }
    return node;
}

struct orc_node *orc_make_tree(float *set, size_t n)
{
    return make_tree((orc_dot *)set, n);
}

void orc_destroy_tree(struct orc_node *tree)
{
    if (!tree) return;
    if (tree->flags & ORC_LEAF) free(tree->data.dots);
    else if (!(tree->flags & ORC_LEAF_MASK))
        for (int i = 0; i < 8; i++) orc_destroy_tree(tree->data.inner.children[i]);
    free(tree);
}

/* ------------------------------------------------------------------ */
/* searches (search.c)                                                 */
/* ------------------------------------------------------------------ */

/* search.c:8-153 */
const struct orc_node *orc_ray(const struct orc_node *tree, const float *origin,
                               const float *dir, float *res, int *slot, orc_counts *cnt)
{
    float bb[3];
    if (!tree) return NULL;
    if (cnt) cnt->nodes++;
    if (!hit_box(&tree->bounding_box, origin, dir, bb)) return NULL;

    if (tree->flags & ORC_DENSE_LEAF) {           /* :31-37 */
        memcpy(res, bb, sizeof(orc_dot));
        if (slot) *slot = 0xFF;
        return tree;
    }
    if (tree->flags & ORC_LEAF) {                 /* :39-81 */
        float closest = INFINITY;
        const struct orc_node *leaf = NULL;
        struct orc_box vox;
        float far[3];
        for (unsigned i = 0; i < tree->dots_num; i++) {
            if (cnt) cnt->voxels++;
            for (int j = 0; j < 3; j++) {
                vox.min[j] = tree->data.dots[i][j];
                vox.max[j] = vox.min[j] + orc_voxel[j];
            }
            if (hit_box(&vox, bb, dir, far)) {
                float d = abs_metric(bb, far);
                if (d == 0) {
                    memcpy(res, far, sizeof(orc_dot));
                    if (slot) *slot = (int)i;
                    return tree;
                }
                if (d < closest) {
                    closest = d;
                    memcpy(res, far, sizeof(orc_dot));
                    if (slot) *slot = (int)i;
                    leaf = tree;
                }
            }
        }
        return leaf;
    }

    if (cnt) cnt->inner++;
    const orc_inner *inner = &tree->data.inner;  /* :84-97 */
    int sub = corrected_subspace_idx(inner->center, bb, dir);
    const struct orc_node *leaf = orc_ray(inner->children[sub], bb, dir, res, slot, cnt);
    if (leaf) return leaf;

    float pi[3][3];                               /* :105-113 */
    int pidx[3];
    unsigned pc = 0;
    for (int i = 0; i < 3; i++) {
        pidx[pc] = i;
        if (hit_plane_within_box(bb, dir, inner->center, i, pi[pc], &tree->bounding_box)) pc++;
    }
    for (unsigned i = 0; i < pc; i++) {           /* :115-148 */
        for (unsigned j = i + 1; j < pc; j++) {
            if (abs_metric(bb, pi[j]) < abs_metric(bb, pi[i])) {
                float t[3];
                memcpy(t, pi[j], sizeof t);
                memcpy(pi[j], pi[i], sizeof t);
                memcpy(pi[i], t, sizeof t);
                int ti = pidx[j]; pidx[j] = pidx[i]; pidx[i] = ti;
            }
        }
        sub ^= 1 << pidx[i];
        leaf = orc_ray(inner->children[sub], pi[i], dir, res, slot, cnt);
        if (leaf) return leaf;
    }
    return NULL;
}

/* search.c:155-183 */
int orc_ball(const struct orc_node *tree, const float *center, float radius, orc_counts *cnt)
{
    if (!tree) return 0;
    if (cnt) cnt->nodes++;
    if (box_ball_interp(&tree->bounding_box, center, radius)) {
        if (tree->flags & ORC_DENSE_LEAF) return 1;
        if (tree->flags & ORC_LEAF) {
            struct orc_box vox;
            for (unsigned i = 0; i < tree->dots_num; i++) {
                if (cnt) cnt->voxels++;
                for (int j = 0; j < 3; j++) {
                    vox.min[j] = tree->data.dots[i][j];
                    vox.max[j] = vox.min[j] + orc_voxel[j];
                }
                if (box_ball_interp(&vox, center, radius)) return 1;
            }
        } else {
            for (int i = 0; i < 8; i++)
                if (orc_ball(tree->data.inner.children[i], center, radius, cnt)) return 1;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ */
/* pre-order numbering                                                 */
/* ------------------------------------------------------------------ */

size_t orc_count_nodes(const struct orc_node *tree)
{
    if (!tree) return 0;
    size_t c = 1;
    if (!(tree->flags & ORC_LEAF_MASK))
        for (int i = 0; i < 8; i++) c += orc_count_nodes(tree->data.inner.children[i]);
    return c;
}

static void preorder_fill(const struct orc_node *t, const struct orc_node **out, size_t *k)
{
    if (!t) return;
    out[(*k)++] = t;
    if (!(t->flags & ORC_LEAF_MASK))
        for (int i = 0; i < 8; i++) preorder_fill(t->data.inner.children[i], out, k);
}

size_t orc_preorder(const struct orc_node *tree, const struct orc_node **out)
{
    size_t k = 0;
    preorder_fill(tree, out, &k);
    return k;
}

typedef struct { const struct orc_node *p; uint32_t id; } ptr_id;

static int cmp_ptr(const void *a, const void *b)
{
    uintptr_t x = (uintptr_t)((const ptr_id *)a)->p, y = (uintptr_t)((const ptr_id *)b)->p;
    return (x > y) - (x < y);
}

static ptr_id *build_index(const struct orc_node *tree, size_t *nn)
{
    size_t n = orc_count_nodes(tree);
    const struct orc_node **pre = malloc((n ? n : 1) * sizeof(*pre));
    orc_preorder(tree, pre);
    ptr_id *idx = malloc((n ? n : 1) * sizeof(ptr_id));
    for (size_t i = 0; i < n; i++) { idx[i].p = pre[i]; idx[i].id = (uint32_t)i; }
    free(pre);
    qsort(idx, n, sizeof(ptr_id), cmp_ptr);
    *nn = n;
    return idx;
}

static uint32_t lookup_id(const ptr_id *idx, size_t n, const struct orc_node *p)
{
    size_t lo = 0, hi = n;
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if ((uintptr_t)idx[mid].p < (uintptr_t)p) lo = mid + 1; else hi = mid;
    }
    return (lo < n && idx[lo].p == p) ? idx[lo].id : UINT32_MAX;
}

/* ------------------------------------------------------------------ */
/* threaded batch drivers                                              */
/* ------------------------------------------------------------------ */

typedef struct {
    size_t n, chunk;
    volatile size_t next;
    pthread_mutex_t mu;
    void (*work)(void *ctx, size_t lo, size_t hi, orc_counts *c);
    void *ctx;
    uint64_t totals[3];
} pool_job;

static void *pool_worker(void *arg)
{
    pool_job *job = arg;
    orc_counts c = {0, 0, 0};
    for (;;) {
        size_t lo = __atomic_fetch_add(&job->next, job->chunk, __ATOMIC_RELAXED);
        if (lo >= job->n) break;
        size_t hi = lo + job->chunk < job->n ? lo + job->chunk : job->n;
        job->work(job->ctx, lo, hi, &c);
    }
    pthread_mutex_lock(&job->mu);
    job->totals[0] += c.nodes; job->totals[1] += c.inner; job->totals[2] += c.voxels;
    pthread_mutex_unlock(&job->mu);
    return NULL;
}

static void run_pool(size_t n, size_t chunk, int nthreads,
                     void (*work)(void *, size_t, size_t, orc_counts *), void *ctx,
                     uint64_t *counts3)
{
    pool_job job;
    job.n = n; job.chunk = chunk ? chunk : 1; job.next = 0;
    job.work = work; job.ctx = ctx;
    job.totals[0] = job.totals[1] = job.totals[2] = 0;
    pthread_mutex_init(&job.mu, NULL);
    if (nthreads < 1) nthreads = 1;
    if (nthreads == 1) {
        pool_worker(&job);
    } else {
        pthread_t *th = malloc(sizeof(pthread_t) * (size_t)nthreads);
        for (int i = 0; i < nthreads; i++) pthread_create(&th[i], NULL, pool_worker, &job);
        for (int i = 0; i < nthreads; i++) pthread_join(th[i], NULL);
        free(th);
    }
    pthread_mutex_destroy(&job.mu);
    if (counts3) { counts3[0] = job.totals[0]; counts3[1] = job.totals[1]; counts3[2] = job.totals[2]; }
}

typedef struct {
    const struct orc_node *root;
    const ptr_id *idx; size_t nidx;
    const float *o, *d;
    uint32_t *leaf; uint8_t *slot; float *pts;
} ray_ctx;

static void ray_work(void *vctx, size_t lo, size_t hi, orc_counts *c)
{
    ray_ctx *x = vctx;
    for (size_t i = lo; i < hi; i++) {
        int s = 0xFF;
        float res[3];
        const struct orc_node *l = orc_ray(x->root, x->o + 3 * i, x->d + 3 * i, res, &s, c);
        if (l) {
            x->leaf[i] = lookup_id(x->idx, x->nidx, l);
            x->slot[i] = (uint8_t)s;
            memcpy(x->pts + 3 * i, res, sizeof res);
        } else {
            x->leaf[i] = UINT32_MAX;
            x->slot[i] = 0xFF;
        }
    }
}

int orc_ray_batch(const struct orc_node *tree, const struct orc_node *root,
                  size_t n, const float *origins, const float *dirs,
                  uint32_t *leaf_id, uint8_t *slot, float *points,
                  uint64_t *counts3, int nthreads)
{
    ray_ctx x;
    x.root = root; x.o = origins; x.d = dirs; x.leaf = leaf_id; x.slot = slot; x.pts = points;
    ptr_id *idx = build_index(tree, &x.nidx);
    x.idx = idx;
    run_pool(n, 4096, nthreads, ray_work, &x, counts3);
    free(idx);
    return 0;
}

typedef struct {
    const struct orc_node *root;
    const float *o, *d;
    uint32_t *per_ray;   /* 3 counters per ray */
} rcount_ctx;

static void rcount_work(void *vctx, size_t lo, size_t hi, orc_counts *c)
{
    rcount_ctx *x = vctx;
    for (size_t i = lo; i < hi; i++) {
        orc_counts k = {0, 0, 0};
        float res[3];
        orc_ray(x->root, x->o + 3 * i, x->d + 3 * i, res, NULL, &k);
        x->per_ray[3 * i] = (uint32_t)k.nodes;
        x->per_ray[3 * i + 1] = (uint32_t)k.inner;
        x->per_ray[3 * i + 2] = (uint32_t)k.voxels;
        c->nodes += k.nodes; c->inner += k.inner; c->voxels += k.voxels;
    }
}

int orc_ray_counts_per_ray(const struct orc_node *root, size_t n, const float *origins,
                           const float *dirs, uint32_t *per_ray, int nthreads)
{
    rcount_ctx x = {root, origins, dirs, per_ray};
    run_pool(n, 4096, nthreads, rcount_work, &x, NULL);
    return 0;
}

typedef struct {
    const struct orc_node *root;
    const float *c, *r;
    uint8_t *hit;
} ball_ctx;

static void ball_work(void *vctx, size_t lo, size_t hi, orc_counts *c)
{
    ball_ctx *x = vctx;
    for (size_t i = lo; i < hi; i++)
        x->hit[i] = (uint8_t)orc_ball(x->root, x->c + 3 * i, x->r[i], c);
}

int orc_ball_batch(const struct orc_node *tree, size_t n, const float *centers,
                   const float *radii, uint8_t *hit, uint64_t *counts3, int nthreads)
{
    ball_ctx x = {tree, centers, radii, hit};
    run_pool(n, 1024, nthreads, ball_work, &x, counts3);
    return 0;
}

/* ------------------------------------------------------------------ */
/* cameras and the render loop                                         */
/* ------------------------------------------------------------------ */

/* vect-ops.c:7-15 */
static void cross(const float *v1, const float *v2, float *r)
{
    float i1 = v1[0], j1 = v1[1], k1 = v1[2];
    float i2 = v2[0], j2 = v2[1], k2 = v2[2];
    r[0] = j1 * k2 - k1 * j2;
    r[1] = -i1 * k2 + k1 * i2;
    r[2] = i1 * j2 - j1 * i2;
}

/* simple-camera.c:21-31 with vect-ops.c:28-36; doom-camera.c:24-57 */
void orc_screen2world(const orc_camera *cam, int sx, int sy, float *ray)
{
    if (cam->kind == 2) {   /* renderer.c:251,260,292: camera->iface->screen2world of another class */
        const float *r = cam->rays + 3 * ((size_t)sy * (size_t)cam->rays_w + (size_t)sx);
        ray[0] = r[0]; ray[1] = r[1]; ray[2] = r[2];
        return;
    }
    if (cam->kind == 1) {
        float d0 = cam->mul * (float)sx - cam->xsub;
        float d1 = 1;
        float d2 = cam->ysub - cam->mul * (float)sy;
        d2 += cam->k;
        ray[0] = d0 * cam->cosphi - d1 * cam->sinphi;
        ray[1] = d1 * cam->cosphi + d0 * cam->sinphi;
        ray[2] = d2;
        return;
    }
    float v[3] = {cam->mul * (float)sx - cam->xsub, 1, cam->ysub - cam->mul * (float)sy};
    float t[3], t2[3];
    cross(cam->rotation + 1, v, t);
    for (int i = 0; i < 3; i++) t[i] = t[i] * 2.0f;
    cross(cam->rotation + 1, t, t2);
    for (int i = 0; i < 3; i++) ray[i] = v[i] + cam->rotation[0] * t[i] + t2[i];
}

/* vect-ops.c:16-24 vox_quat_mul: res = q1 * q2 (res may alias either). */
static void quat_mul(const float *q1, const float *q2, float *res)
{
    float e1 = q1[0], i1 = q1[1], j1 = q1[2], k1 = q1[3];
    float e2 = q2[0], i2 = q2[1], j2 = q2[2], k2 = q2[3];
    res[0] = e1 * e2 - i1 * i2 - j1 * j2 - k1 * k2;
    res[1] = j1 * k2 - k1 * j2 + i1 * e2 + e1 * i2;
    res[2] = k1 * i2 - i1 * k2 + j1 * e2 + e1 * j2;
    res[3] = i1 * j2 - j1 * i2 + k1 * e2 + e1 * k2;
}

/* vect-ops.c:38-46 vox_rotate_vector_q: the vector part of `v` rotated by
 * `q` into res[1..3]; res[0] is left alone. */
static void rotate_vector_q(const float *q, const float *v, float *res)
{
    float t[3], t2[3];
    cross(q + 1, v + 1, t);
    for (int i = 0; i < 3; i++) t[i] = t[i] * 2.0f;
    cross(q + 1, t, t2);
    for (int i = 0; i < 3; i++) res[i + 1] = v[i + 1] + q[0] * t[i] + t2[i];
}

/* A simple-camera as vox_simple_camera_construct, set_property_number("fov"),
 * set_window_size, set_property_dot("position") and look_at leave it
 * (simple-camera.c:139-159, :161-165, :120-136, :167-170, :106-118 with
 * simple_rotate_camera :50-99 and vect-ops.c:48-58 vox_quat_normalize).
 * Host-side set-up only: the renderer reads the resulting fields. */
void orc_camera_simple(orc_camera *cam, const float position[3], const float target[3], int w, int h, float fov)
{
    memset(cam, 0, sizeof *cam);
    cam->kind = 0;
    if (w > h) {                                  /* simple-camera.c:124-135 */
        cam->xsub = fov;
        cam->ysub = fov * h / w;
        cam->mul = fov * 2 / w;
    } else {
        cam->ysub = fov;
        cam->xsub = fov * w / h;
        cam->mul = fov * 2 / h;
    }
    for (int i = 0; i < 3; i++) cam->position[i] = position[i];
    float *q = cam->rotation;
    q[0] = 1.0f; q[1] = q[2] = q[3] = 0.0f;       /* vox_quat_set_identity */
    float sub[3], rot[3];
    for (int i = 0; i < 3; i++) sub[i] = target[i] - cam->position[i];
    rot[0] = atan2f(sub[2], hypotf(sub[0], sub[1]));
    rot[1] = 0;
    rot[2] = -atan2f(sub[0], sub[1]);
    static const float orts[3][4] = {{0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
    for (int i = 2; i >= 0; i--) {                /* z, then y, then x axis of the camera */
        float r[4];
        rotate_vector_q(q, orts[i], r);
        float s = sinf(rot[i] / 2), c = cosf(rot[i] / 2);
        for (int j = 0; j < 3; j++) r[j + 1] = s * r[j + 1];
        r[0] = c;
        quat_mul(r, q, q);
    }
    float sum = 0;
    for (int i = 0; i < 4; i++) sum += q[i] * q[i];
    float norm = sqrtf(sum);
    for (int i = 0; i < 4; i++) q[i] /= norm;
}

/* ------------------------------------------------------------------ */
/* light manager and its M-tree (src/voxrnd/lights.c,                  */
/* src/voxtrees/mtree.c), restated recursively as the reference has it  */
/* ------------------------------------------------------------------ */

#define ORC_MT_MAX 9                                  /* mtree.h:44 */

typedef struct {                                      /* mtree.h:17-40 */
    float center[3], color[3], radius, sqr_radius;
} orc_sphere;

typedef struct orc_mt {                               /* mtree.h:46-56 */
    orc_sphere bs;
    struct orc_mt *parent;
    unsigned leaf, num;
    struct orc_mt *children[ORC_MT_MAX + 1];
    orc_sphere *spheres;
} orc_mt;

struct orc_lights {                                   /* lights.c:11-14 */
    float ambient[3];
    orc_mt *root;
};

static orc_mt *mt_alloc(int leaf)                     /* mtree.c:11-19 */
{
    orc_mt *n = calloc(1, sizeof *n);
    n->leaf = leaf;
    if (leaf) n->spheres = calloc(ORC_MT_MAX + 1, sizeof(orc_sphere));
    return n;
}

static const orc_sphere *mt_item(const orc_mt *n, unsigned i)
{
    return n->leaf ? &n->spheres[i] : &n->children[i]->bs;
}

static int mt_bounding(const orc_sphere *s, orc_sphere *b)   /* mtree.c:21-56, scalar branch */
{
    float dist = sqrtf(sqr_metric(s->center, b->center));
    float crit = (1 + (b->radius - s->radius) / dist) / 2;
    int changed = 1;
    if (crit < 0) {
        *b = *s;
    } else if (crit < 1) {
        b->radius = (s->radius + b->radius + dist) / 2;
        b->sqr_radius = pow(b->radius, 2);
        for (int i = 0; i < 3; i++) b->center[i] = b->center[i] - s->center[i];   /* vox_dot_sub */
        for (int i = 0; i < 3; i++) b->center[i] = crit * b->center[i];           /* vox_dot_scmul */
        for (int i = 0; i < 3; i++) b->center[i] = b->center[i] + s->center[i];   /* vox_dot_add */
    } else {
        changed = 0;
    }
    return changed;
}

static int mt_node_bounding(orc_mt *n)                /* mtree.c:58-74 */
{
    int changed = 0;
    n->bs = *mt_item(n, 0);
    for (unsigned i = 1; i < n->num; i++) changed += mt_bounding(mt_item(n, i), &n->bs);
    return !!changed;
}

static void mt_propagate(orc_mt *n)                   /* mtree.c:76-87 */
{
    if (n != NULL && mt_node_bounding(n)) mt_propagate(n->parent);
}

static orc_mt *mt_split(orc_mt *n)                    /* mtree.c:89-180 */
{
    float c1[3], c2[3], maxd = 0;
    memcpy(c1, mt_item(n, 0)->center, 12);            /* defined when all centres coincide */
    memcpy(c2, mt_item(n, 0)->center, 12);
    for (unsigned i = 0; i < n->num; i++)
        for (unsigned j = i + 1; j < n->num; j++) {
            float d = sqr_metric(mt_item(n, i)->center, mt_item(n, j)->center);
            if (d > maxd) { memcpy(c1, mt_item(n, i)->center, 12); memcpy(c2, mt_item(n, j)->center, 12); maxd = d; }
        }
    orc_mt *parent = n->parent, *res = parent;
    orc_mt *n1 = mt_alloc(n->leaf), *n2 = mt_alloc(n->leaf);
    n1->parent = n2->parent = parent;
    for (unsigned i = 0; i < n->num; i++) {
        float d1 = sqr_metric(mt_item(n, i)->center, c1), d2 = sqr_metric(mt_item(n, i)->center, c2);
        orc_mt *w = d1 < d2 ? n1 : n2;
        if (n->leaf) w->spheres[w->num] = n->spheres[i];
        else { w->children[w->num] = n->children[i]; n->children[i]->parent = w; }
        w->num++;
    }
    mt_node_bounding(n1);
    mt_node_bounding(n2);
    if (parent) {
        for (unsigned i = 0; i < parent->num; i++)
            if (parent->children[i] == n) parent->children[i] = n1;
        parent->children[parent->num++] = n2;
        mt_propagate(parent);
        if (parent->num == ORC_MT_MAX + 1) res = mt_split(parent);
    } else {
        res = mt_alloc(0);
        res->num = 2;
        res->children[0] = n1;
        res->children[1] = n2;
        mt_node_bounding(res);
        n1->parent = n2->parent = res;
    }
    free(n->spheres);
    free(n);
    return res;
}

static orc_mt *mt_contains(orc_mt *n, const orc_sphere *s)   /* mtree.c:182-216 */
{
    if (n == NULL || !(sqr_metric(s->center, n->bs.center) < n->bs.sqr_radius)) return NULL;
    if (n->leaf) {
        for (unsigned i = 0; i < n->num; i++)
            if (memcmp(n->spheres[i].center, s->center, 12) == 0 && n->spheres[i].radius == s->radius) return n;
        return NULL;
    }
    for (unsigned i = 0; i < n->num; i++) {
        orc_mt *r = mt_contains(n->children[i], s);
        if (r) return r;
    }
    return NULL;
}

static orc_mt *mt_add(orc_mt *n, const orc_sphere *s)        /* mtree.c:218-253 */
{
    orc_mt *res = n;
    float sqr_radius = pow(s->radius, 2);
    if (n == NULL) {
        res = mt_alloc(1);
        res->bs = *s;
        res->bs.sqr_radius = sqr_radius;
        res->num = 1;
        res->spheres[0] = *s;
        res->spheres[0].sqr_radius = sqr_radius;
    } else if (n->leaf) {
        n->spheres[n->num] = *s;
        n->spheres[n->num].sqr_radius = sqr_radius;
        n->num++;
        mt_propagate(n);
        if (n->num == ORC_MT_MAX + 1) res = mt_split(n);
    } else {
        orc_mt *child = n->children[0];
        float mind = INFINITY;
        for (unsigned i = 0; i < n->num; i++) {
            float d = sqr_metric(s->center, n->children[i]->bs.center);
            if (d < mind) { mind = d; child = n->children[i]; }
        }
        res = mt_add(child, s);
    }
    return res;
}

static void mt_free(orc_mt *n)
{
    if (!n) return;
    if (n->leaf) free(n->spheres);
    else for (unsigned i = 0; i < n->num; i++) mt_free(n->children[i]);
    free(n);
}

static orc_mt *mt_delete_leaf(orc_mt *n)              /* mtree.c:269-322 */
{
    orc_mt *parent = n->parent;
    mt_free(n);
    if (parent == NULL) return NULL;
    unsigned i;
    for (i = 0; i < parent->num; i++)
        if (parent->children[i] == n) break;
    if (parent->num == 2) {
        orc_mt *other = parent->children[1 - i], *top = parent->parent;
        free(parent);
        other->parent = top;
        if (top == NULL) return other;
        for (i = 0; i < top->num; i++)
            if (top->children[i] == parent) break;
        top->children[i] = other;
        mt_propagate(top);
        return top;
    }
    parent->num--;
    memmove(&parent->children[i], &parent->children[i + 1], sizeof(orc_mt *) * (parent->num - i));
    parent->children[parent->num] = NULL;
    mt_propagate(parent);
    return parent;
}

orc_lights *orc_lights_new(void)                      /* lights.c:16-23 */
{
    orc_lights *l = calloc(1, sizeof *l);
    l->ambient[0] = l->ambient[1] = l->ambient[2] = 1;
    return l;
}

void orc_lights_free(orc_lights *l)
{
    if (!l) return;
    mt_free(l->root);
    free(l);
}

static int valid_light(const float *c)                /* lights.c:81-89 */
{
    for (int i = 0; i < 3; i++)
        if (c[i] < 0 || c[i] > 1) return 0;
    return 1;
}

int orc_lights_ambient(orc_lights *l, const float *color)
{
    if (!valid_light(color)) return 0;
    memcpy(l->ambient, color, 12);
    return 1;
}

int orc_lights_insert(orc_lights *l, const float *center, float radius, const float *color)
{
    if (!valid_light(color)) return 0;                /* lights.c:46-58 */
    orc_sphere s;
    memset(&s, 0, sizeof s);
    memcpy(s.center, center, 12);
    memcpy(s.color, color, 12);
    s.radius = radius;
    if (!(s.radius > 0) || mt_contains(l->root, &s)) return 0;   /* mtree.c:255-267 */
    orc_mt *n = mt_add(l->root, &s);
    if (n->parent == NULL) l->root = n;
    return 1;
}

int orc_lights_delete(orc_lights *l, const float *center, float radius)
{
    orc_sphere s;                                     /* lights.c:60-68, mtree.c:324-368 */
    memset(&s, 0, sizeof s);
    memcpy(s.center, center, 12);
    s.radius = radius;
    orc_mt *leaf = mt_contains(l->root, &s);
    if (!(s.radius > 0) || leaf == NULL) return 0;
    orc_mt *last = leaf;
    if (leaf->num == 1) {
        last = mt_delete_leaf(leaf);
    } else {
        unsigned i;
        for (i = 0; i < leaf->num; i++)
            if (memcmp(leaf->spheres[i].center, s.center, 12) == 0 && leaf->spheres[i].radius == s.radius) break;
        memmove(&leaf->spheres[i], &leaf->spheres[i + 1], sizeof(orc_sphere) * (leaf->num - i - 1));
        leaf->num--;
        mt_propagate(leaf);
    }
    if (last == NULL || last->parent == NULL) l->root = last;
    return 1;
}

static unsigned mt_items(const orc_mt *n)
{
    if (!n) return 0;
    if (n->leaf) return n->num;
    unsigned c = 0;
    for (unsigned i = 0; i < n->num; i++) c += mt_items(n->children[i]);
    return c;
}

int orc_lights_count(const orc_lights *l) { return (int)mt_items(l->root); }

typedef struct { float inter[3], color[3]; int n; } light_acc;

static void light_cb(const orc_sphere *s, light_acc *a)   /* lights.c:91-102 */
{
    float dist = fminf(s->radius, sqrtf(sqr_metric(s->center, a->inter)));
    float add = 1 - dist / s->radius;
    a->color[0] = a->color[0] + add * s->color[0];
    a->color[1] = a->color[1] + add * s->color[1];
    a->color[2] = a->color[2] + add * s->color[2];
    a->n++;
}

static void mt_search(const orc_mt *n, light_acc *a)   /* mtree.c:463-493 */
{
    if (n == NULL || !(sqr_metric(n->bs.center, a->inter) < n->bs.sqr_radius)) return;
    if (n->leaf) {
        if (n->num == 1) { light_cb(&n->spheres[0], a); return; }
        for (unsigned i = 0; i < n->num; i++)
            if (sqr_metric(n->spheres[i].center, a->inter) < n->spheres[i].sqr_radius) light_cb(&n->spheres[i], a);
        return;
    }
    for (unsigned i = 0; i < n->num; i++) mt_search(n->children[i], a);
}

int orc_lights_get(const orc_lights *l, const float *p, float *light)   /* lights.c:104-116 */
{
    light_acc a;
    memcpy(a.inter, p, 12);
    memcpy(a.color, l->ambient, 12);
    a.n = 0;
    mt_search(l->root, &a);
    memcpy(light, a.color, 12);
    return a.n;
}

/* The reference's own M-tree invariants (tests/tests.c:779-808): at most
 * MAX items a node, inner nodes with two or more children whose parent link
 * points back, every item inside its node's bounding sphere within 0.5.
 * Returns 0 when they hold. */
static int mt_verify(const orc_mt *n)
{
    if (!n) return 0;
    if (n->num > ORC_MT_MAX) return 1;
    for (unsigned i = 0; i < n->num; i++) {
        const orc_sphere *s = mt_item(n, i);
        float dist = sqrtf(sqr_metric(s->center, n->bs.center));
        if (!(s->radius + dist < n->bs.radius + 0.5f)) return 2;
        if (!n->leaf) {
            if (n->num < 2 || n->children[i] == NULL || n->children[i]->parent != n) return 3;
            if (mt_verify(n->children[i])) return 4;
        }
    }
    return 0;
}

int orc_lights_verify(const orc_lights *l) { return mt_verify(l->root); }

/* renderer.c:27-52 get_color; SDL_MapRGB on ARGB8888.  Without a light
 * manager the texel is grey; with one, min(light, 1) * texel per channel,
 * converted to 8 bits as C converts a float to Uint8 (truncation). */
static uint32_t get_color_lit(const uint8_t *tex, const orc_lights *lights, const float *inter)
{
    int x = abs((int)(inter[0] / orc_voxel[0])) & 31;
    int y = abs((int)(inter[1] / orc_voxel[1])) & 31;
    int z = abs((int)(inter[2] / orc_voxel[2])) & 31;
    uint8_t c = tex[x * 1024 + y * 32 + z];
    if (lights == NULL) return 0xFF000000u | ((uint32_t)c << 16) | ((uint32_t)c << 8) | c;
    float light[3];
    orc_lights_get(lights, inter, light);
    uint8_t r = fminf(light[0], 1.0) * c;
    uint8_t g = fminf(light[1], 1.0) * c;
    uint8_t b = fminf(light[2], 1.0) * c;
    return 0xFF000000u | ((uint32_t)r << 16) | ((uint32_t)g << 8) | b;
}

static uint32_t get_color(const uint8_t *tex, const float *inter) { return get_color_lit(tex, NULL, inter); }

static const int zorder[16] = {0, 1, 4, 5, 2, 3, 6, 7, 8, 9, 12, 13, 10, 11, 14, 15}; /* renderer.c:23-25 */

typedef struct {
    const struct orc_node *tree;
    const orc_camera *cam;
    int w, ws;
    const uint8_t *tex;
    uint32_t *argb;
} render_ctx;

static void render_work(void *vctx, size_t lo, size_t hi, orc_counts *c)
{
    render_ctx *x = vctx;
    for (size_t cs = lo; cs < hi; cs++) {
        int ys = (int)(cs / (size_t)x->ws) * 4, xs = (int)(cs % (size_t)x->ws) * 4;
        for (int i = 0; i < 16; i++) {
            int p = zorder[i], px = xs + p % 4, py = ys + p / 4;
            float dir[3], inter[3];
            orc_screen2world(x->cam, px, py, dir);
            const struct orc_node *l = orc_ray(x->tree, x->cam->position, dir, inter, NULL, c);
            x->argb[(size_t)py * x->w + px] = l ? get_color(x->tex, inter) : 0u;
        }
    }
}

int orc_render_best(const struct orc_node *tree, const orc_camera *cam,
                    int w, int h, const uint8_t *texture, uint32_t *argb,
                    uint64_t *counts3, int nthreads)
{
    if ((w & 0xf) || (h & 0x3)) return -1;   /* renderer.c:97-100 bad_geometry */
    render_ctx x = {tree, cam, w, w / 4, texture, argb};
    run_pool((size_t)(w / 4) * (size_t)(h / 4), 64, nthreads, render_work, &x, counts3);
    return 0;
}

/* renderer.c:215-318 for any quality: per 4x4 square, Z-order, FAST leaf
 * reuse, ADAPTIVE corner test, ray merging.  Undrawn pixels stay 0. */
typedef struct {
    const struct orc_node *tree;
    const orc_camera *cam;
    int w, ws;
    unsigned quality;
    const uint8_t *tex;
    uint32_t *argb;
    const orc_lights *lights;
} quality_ctx;

static float sqr_norm(const float *a)
{
    float r = 0;
    for (int i = 0; i < 3; i++) r += a[i] * a[i];
    return r;
}

static void quality_work(void *vctx, size_t lo, size_t hi, orc_counts *c)
{
    quality_ctx *x = vctx;
    int rnd_mode = x->quality & 3, merge_mode = x->quality & 12;
    const float *origin = x->cam->position;
    for (size_t cs = lo; cs < hi; cs++) {
        int ystart = (int)(cs / (size_t)x->ws) * 4, xstart = (int)(cs % (size_t)x->ws) * 4;
        uint32_t out[16] = {0};
        const struct orc_node *leaf = NULL;
        float dir1[3], dir2[3], inter1[3], inter2[3];
        int block_mode = rnd_mode, istart = 0, iend = 16, block_merge = 0;
        if (block_mode == 2) {
            block_merge = (merge_mode == 4);
            istart = 1;
            orc_screen2world(x->cam, xstart, ystart, dir1);
            const struct orc_node *c1 = orc_ray(x->tree, origin, dir1, inter1, NULL, c);
            block_mode = 1;
            leaf = c1;
            if (c1) {
                iend = 15;
                out[0] = get_color_lit(x->tex, x->lights, inter1);
                orc_screen2world(x->cam, xstart + 3, ystart + 3, dir2);
                const struct orc_node *c2 = orc_ray(x->tree, origin, dir2, inter2, NULL, c);
                if (c2) {
                    out[15] = get_color_lit(x->tex, x->lights, inter2);
                    float d1 = sqr_metric(inter1, origin);
                    float d2 = sqr_norm(dir1);
                    float criteria = d1 / d2 * sqr_metric(dir1, dir2);
                    float dist = sqr_metric(inter1, inter2);
                    if (dist / criteria > 1.69) block_mode = 0;
                    if (d1 > 150 * 150)
                        block_merge = (block_mode == 1 && merge_mode == 8) ? 1 : block_merge;
                    else
                        block_merge = 0;
                }
            }
        }
        int prev_p = 0;
        for (int i = istart; i < iend; i++) {
            int p = zorder[i];
            int merge = block_merge && (i & 1);
            orc_screen2world(x->cam, p % 4 + xstart, p / 4 + ystart, dir1);
            if (!merge) {
                if (block_mode == 1) {
                    if (leaf) leaf = orc_ray(leaf, origin, dir1, inter1, NULL, c);
                    if (!leaf) leaf = orc_ray(x->tree, origin, dir1, inter1, NULL, c);
                } else {
                    leaf = orc_ray(x->tree, origin, dir1, inter1, NULL, c);
                }
            }
            if (leaf) out[p] = merge ? out[prev_p] : get_color_lit(x->tex, x->lights, inter1);
            prev_p = p;
        }
        for (int i = 0; i < 16; i++)
            x->argb[(size_t)(ystart + i / 4) * x->w + xstart + i % 4] = out[i];
    }
}

int orc_render_quality(const struct orc_node *tree, const orc_camera *cam, int w, int h,
                       unsigned quality, const uint8_t *texture, uint32_t *argb,
                       uint64_t *counts3, int nthreads)
{
    if ((w & 0xf) || (h & 0x3)) return -1;
    quality_ctx x = {tree, cam, w, w / 4, quality, texture, argb, NULL};
    run_pool((size_t)(w / 4) * (size_t)(h / 4), 64, nthreads, quality_work, &x, counts3);
    return 0;
}

int orc_render_lit(const struct orc_node *tree, const orc_camera *cam, int w, int h, unsigned quality,
                   const uint8_t *texture, const orc_lights *lights, uint32_t *argb, int nthreads)
{
    if ((w & 0xf) || (h & 0x3)) return -1;
    quality_ctx x = {tree, cam, w, w / 4, quality, texture, argb, lights};
    run_pool((size_t)(w / 4) * (size_t)(h / 4), 64, nthreads, quality_work, &x, NULL);
    return 0;
}

/* ------------------------------------------------------------------ */
/* dumps                                                               */
/* ------------------------------------------------------------------ */

size_t orc_count_stored_dots(const struct orc_node *tree)
{
    if (!tree) return 0;
    if (tree->flags & ORC_DENSE_LEAF) return 0;
    if (tree->flags & ORC_LEAF) return tree->dots_num;
    size_t c = 0;
    for (int i = 0; i < 8; i++) c += orc_count_stored_dots(tree->data.inner.children[i]);
    return c;
}

typedef struct {
    uint32_t *flags, *dots_num; float *boxes, *centers; uint8_t *mask;
    uint64_t *doff; float *dots; size_t k, nd;
} dump_ctx;

static void dump_rec(const struct orc_node *t, dump_ctx *d)
{
    if (!t) return;
    size_t k = d->k++;
    d->flags[k] = t->flags;
    d->dots_num[k] = t->dots_num;
    memcpy(d->boxes + 6 * k, &t->bounding_box, 6 * sizeof(float));
    memset(d->centers + 3 * k, 0, 3 * sizeof(float));
    d->mask[k] = 0;
    d->doff[k] = d->nd;
    if (t->flags & ORC_DENSE_LEAF) return;
    if (t->flags & ORC_LEAF) {
        memcpy(d->dots + 3 * d->nd, t->data.dots, t->dots_num * sizeof(orc_dot));
        d->nd += t->dots_num;
        return;
    }
    memcpy(d->centers + 3 * k, t->data.inner.center, 3 * sizeof(float));
    for (int i = 0; i < 8; i++)
        if (t->data.inner.children[i]) d->mask[k] |= (uint8_t)(1u << i);
    for (int i = 0; i < 8; i++) dump_rec(t->data.inner.children[i], d);
}

size_t orc_dump(const struct orc_node *tree, uint32_t *flags, uint32_t *dots_num,
                float *boxes, float *centers, uint8_t *child_mask,
                uint64_t *dot_offset, float *dots)
{
    dump_ctx d = {flags, dots_num, boxes, centers, child_mask, dot_offset, dots, 0, 0};
    dump_rec(tree, &d);
    return d.k;
}

typedef struct {
    const uint32_t *flags, *dots_num; const float *boxes, *centers; const uint8_t *mask;
    const uint64_t *doff; const float *dots; size_t k, n;
} undump_ctx;

static struct orc_node *undump_rec(undump_ctx *u)
{
    if (u->k >= u->n) return NULL;
    size_t k = u->k++;
    struct orc_node *t = calloc(1, sizeof(struct orc_node));
    t->flags = u->flags[k];
    t->dots_num = u->dots_num[k];
    memcpy(&t->bounding_box, u->boxes + 6 * k, 6 * sizeof(float));
    if (t->flags & ORC_DENSE_LEAF) return t;
    if (t->flags & ORC_LEAF) {
        size_t cap = t->dots_num > ORC_MAX_DOTS ? t->dots_num : ORC_MAX_DOTS;
        t->data.dots = malloc(cap * sizeof(orc_dot));
        memcpy(t->data.dots, u->dots + 3 * u->doff[k], t->dots_num * sizeof(orc_dot));
        return t;
    }
    memcpy(t->data.inner.center, u->centers + 3 * k, 3 * sizeof(float));
    uint8_t m = u->mask[k];
    for (int i = 0; i < 8; i++)
        t->data.inner.children[i] = (m >> i & 1) ? undump_rec(u) : NULL;
    return t;
}

struct orc_node *orc_from_dump(size_t nnodes, const uint32_t *flags,
                               const uint32_t *dots_num, const float *boxes,
                               const float *centers, const uint8_t *child_mask,
                               const uint64_t *dot_offset, const float *dots)
{
    undump_ctx u = {flags, dots_num, boxes, centers, child_mask, dot_offset, dots, 0, nnodes};
    return nnodes ? undump_rec(&u) : NULL;
}
