/*
 * traverse.cuh -- device-side voxtrees searches over the pool of
 * pool_layout.h.
 *
 * Exactness.  Every float operation the reference performs is performed
 * here, in the same order, with the IEEE round-to-nearest intrinsics
 * (__fadd_rn, __fsub_rn, __fmul_rn, __fdiv_rn), which the compiler never
 * contracts into FMAs.  Comparisons keep the reference's NaN behaviour.  The
 * result is the reference's leaf, voxel and intersection point, bit for bit.
 *
 * Recursion becomes an explicit per-thread stack of pending tasks {record
 * offset, ray origin} (see trace_ray).
 *
 * Checked build (-DVOX_CUDA_CHECKED, libvoxtrees_cuda_checked.so): every
 * load from the tree image and the light tree first proves its index inside
 * the uploaded arrays; an index outside marks the tree's status word with
 * VOX_STATUS_RANGE and ends that search as an error instead of reading.  It
 * stands in for a memory checker on the search kernels; the normal build
 * relies on the upload-time validation of the image instead.
 */
#ifndef VOX_TRAVERSE_CUH
#define VOX_TRAVERSE_CUH

#include <cstdint>
#include <cuda_runtime.h>

#include "pool_layout.h"
#include "../../include/voxtrees_cuda.h"

namespace vox {

struct DevTree {
    const uint4 *pool;
    const uint32_t *rec_of_id;   // pre-order id -> record offset
    uint32_t root;               // record offset of the root, VOXP_EMPTY if none
    uint32_t n_nodes;
    float vx, vy, vz;            // vox_voxel at upload time
    uint32_t max_steps;          // nodes + voxels: no search takes more loop steps
    uint32_t n_units;            // 16-byte units in the image (pool)
    uint32_t *fault;             // the tree's status word (checked build only)
};

struct Counts {
    uint32_t nodes, inner, voxels;
};

// Status word bits: a search ran out of stack or steps; (checked build) an
// index outside the uploaded arrays.
constexpr uint32_t VOX_STATUS_STACK = 1u, VOX_STATUS_RANGE = 2u;

#ifdef VOX_CUDA_CHECKED
constexpr bool CHECKED = true;
#else
constexpr bool CHECKED = false;
#endif

// Units [at, at + span) lie in an array of n units; without the checked
// build always true (and compiled away).  Marks `fault` when not.
__device__ __forceinline__ bool in_range(uint64_t at, uint32_t span, uint64_t n, uint32_t *fault)
{
    if (!CHECKED) return true;
    if (at + span <= n) return true;
    if (fault) atomicOr(fault, VOX_STATUS_RANGE);
    return false;
}

__device__ __forceinline__ float ubf(uint32_t u) { return __uint_as_float(u); }

__device__ __forceinline__ uint4 ld16(const uint4 *p) { return __ldg(p); }

/* geom.c:13-31 + :69-99 (hit_box).  Returns the entry point of the ray into
 * the closed box [lo, hi] in r.  An axis on which the origin already lies
 * inside the slab yields a distance of +-0 or NaN in the reference, which can
 * never be the winning positive distance, so only clamped axes divide. */
__device__ __forceinline__ bool hit_box(float lx, float ly, float lz, float hx, float hy, float hz,
                                        float ox, float oy, float oz, float dx, float dy, float dz,
                                        float &rx, float &ry, float &rz)
{
    bool cx = true, cy = true, cz = true;
    rx = ox; ry = oy; rz = oz;
    if (ox < lx) rx = lx; else if (ox > hx) rx = hx; else cx = false;
    if (oy < ly) ry = ly; else if (oy > hy) ry = hy; else cy = false;
    if (oz < lz) rz = lz; else if (oz > hz) rz = hz; else cz = false;
    if (!(cx | cy | cz)) return true;

    int plane = -1;
    float maxd = -1.0f;
    if (cx) { float t = __fdiv_rn(__fsub_rn(rx, ox), dx); if (t > maxd) { plane = 0; maxd = t; } }
    if (cy) { float t = __fdiv_rn(__fsub_rn(ry, oy), dy); if (t > maxd) { plane = 1; maxd = t; } }
    if (cz) { float t = __fdiv_rn(__fsub_rn(rz, oz), dz); if (t > maxd) { plane = 2; maxd = t; } }
    if (maxd <= 0.0f) return false;

    if (plane != 0) {
        float t = __fadd_rn(ox, __fmul_rn(maxd, dx));
        if (t < lx || t > hx) return false;
        rx = t;
    }
    if (plane != 1) {
        float t = __fadd_rn(oy, __fmul_rn(maxd, dy));
        if (t < ly || t > hy) return false;
        ry = t;
    }
    if (plane != 2) {
        float t = __fadd_rn(oz, __fmul_rn(maxd, dz));
        if (t < lz || t > hz) return false;
        rz = t;
    }
    return true;
}

/* geom.c:125-131 vox_abs_metric: ((|dx| + |dy|) + |dz|). */
__device__ __forceinline__ float l1(float ax, float ay, float az, float bx, float by, float bz)
{
    return __fadd_rn(__fadd_rn(fabsf(__fsub_rn(ax, bx)), fabsf(__fsub_rn(ay, by))),
                     fabsf(__fsub_rn(az, bz)));
}

/* geom.c:101-123 hit_plane_within_box for axis p.  Every comparison is made
 * and combined, with no early exit: the answer is the reference's (its point
 * is used only when the answer is true), and the lanes of a warp take no
 * branch here.  Measured: per-frame BEST launches 15% faster than with the
 * reference's early returns, the persistent batch kernel 2.6%. */
__device__ __forceinline__ bool hit_plane(int p, float ox, float oy, float oz, float dx, float dy, float dz,
                                          float cp, float lx, float ly, float lz, float hx, float hy, float hz,
                                          float &rx, float &ry, float &rz)
{
    float op = p == 0 ? ox : (p == 1 ? oy : oz);
    float dp = p == 0 ? dx : (p == 1 ? dy : dz);
    float k = __fsub_rn(cp, op);
    bool ok = !(k == 0.0f || ((dp < 0.0f) != (k < 0.0f)));
    k = __fdiv_rn(k, dp);
    rx = __fadd_rn(ox, __fmul_rn(k, dx));
    ry = __fadd_rn(oy, __fmul_rn(k, dy));
    rz = __fadd_rn(oz, __fmul_rn(k, dz));
    // NaN coordinates pass, as the reference's `<` / `>` tests let them
    ok &= !(rx < lx) & !(rx > hx) & !(ry < ly) & !(ry > hy) & !(rz < lz) & !(rz > hz);
    return ok;
}

struct RayHit {
    float x, y, z;
    uint32_t leaf;    // pre-order id
    uint32_t slot;    // winning voxel, 0xFF for dense
    uint32_t rec;     // record offset of the leaf
};

/* vox_ray_tree_intersection (search.c:8-153) as a resumable search.
 *
 * RaySearch holds everything one search carries between loop iterations
 * except its stack of pending tasks, which the caller keeps beside it (a
 * separate local array, so the search state itself stays in registers), and
 * ray_step() runs one iteration.  Every iteration makes one 16..48-byte load
 * (a node record, or one voxel of the leaf being scanned) and one box test,
 * so the lanes of a warp stay in step whatever mix of nodes and voxels they
 * are on, and a lane whose search ended could start another between any
 * two iterations.  The box test of a node is
 * search.c:22-23; of a voxel, the leaf loop's test at :55.  When an inner
 * node's box is entered, its plane crossings (:105-148) are computed at once:
 * the children behind the crossings are pushed in visiting order and the
 * search continues in the entry octant (:86-97).  Computing the crossings
 * before the entry octant has been searched changes nothing: they depend only
 * on the node and the ray, and they are used only if that octant finds
 * nothing.  The first hit ends the search, as the first non-NULL return ends
 * the recursion.
 *
 * The stack holds pending tasks {record offset, ray origin}; it never needs
 * more than 3 entries per inner level, which the upload-time depth check
 * guarantees for CAP.  A search that would overflow it, or that takes more
 * iterations than the tree has nodes and voxels (a damaged pool), ends with
 * STEP_ERROR. */
enum : int { STEP_MORE = 0, STEP_HIT = 1, STEP_MISS = 2, STEP_ERROR = 3 };

struct RaySearch {
    int sp;                    // entries on the caller's stack
    uint32_t cur;              // node mode: record offset; voxel mode: first voxel
    float ox, oy, oz;          // origin of the next box test
    float dx, dy, dz;
    bool scan;                 // scanning the voxels of a leaf
    uint32_t vi, vn, vrec, vid;
    float best, bx, by, bz;
    int win;
    uint32_t steps;
};

__device__ __forceinline__ void ray_begin(RaySearch &s, uint32_t start, float ox, float oy, float oz,
                                          float dx, float dy, float dz)
{
    s.sp = 0;
    s.cur = start;
    s.ox = ox; s.oy = oy; s.oz = oz;
    s.dx = dx; s.dy = dy; s.dz = dz;
    s.scan = false;
    s.vi = 0; s.vn = 0; s.vrec = 0; s.vid = 0;
    s.best = 0.0f; s.bx = 0.0f; s.by = 0.0f; s.bz = 0.0f;
    s.win = -1;
    s.steps = 0;
}

/* search.c:105-148: the crossings of the ray (from the entry point e of an
 * inner node) with the node's three dividing planes that lie in its box,
 * sorted by L1 distance from e with the reference's selection sort
 * (:115-134, immediate swaps on '<'); each crossing flips one octant bit of
 * the entry octant `sub` (:137).  Pushes the crossing children so that they
 * pop in visiting order (NULL children are skipped: they return NULL at
 * once).  Returns false when the stack would overflow. */
template <int CAP>
__device__ __forceinline__ bool push_crossings(RaySearch &s, uint4 (&stack)[CAP], float ex, float ey, float ez,
                                               float lx, float ly, float lz, float hx, float hy, float hz,
                                               float cx, float cy, float cz, uint32_t sub, uint32_t mask,
                                               uint32_t link)
{
    const float dx = s.dx, dy = s.dy, dz = s.dz;
    float qx0, qy0, qz0, qx1, qy1, qz1, qx2, qy2, qz2;
    bool v0 = hit_plane(0, ex, ey, ez, dx, dy, dz, cx, lx, ly, lz, hx, hy, hz, qx0, qy0, qz0);
    bool v1 = hit_plane(1, ex, ey, ez, dx, dy, dz, cy, lx, ly, lz, hx, hy, hz, qx1, qy1, qz1);
    bool v2 = hit_plane(2, ex, ey, ez, dx, dy, dz, cz, lx, ly, lz, hx, hy, hz, qx2, qy2, qz2);
    int pc = (int)v0 + (int)v1 + (int)v2;
    // compacted slots a, b, c = first, second, third valid crossing
    float ax = v0 ? qx0 : (v1 ? qx1 : qx2);
    float ay = v0 ? qy0 : (v1 ? qy1 : qy2);
    float az = v0 ? qz0 : (v1 ? qz1 : qz2);
    int ai = v0 ? 0 : (v1 ? 1 : 2);
    bool ab1 = v0 && v1;
    float bxp = ab1 ? qx1 : qx2, byp = ab1 ? qy1 : qy2, bzp = ab1 ? qz1 : qz2;
    int bi = ab1 ? 1 : 2;
    float cxp = qx2, cyp = qy2, czp = qz2;
    int ci = 2;
    float ma = l1(ex, ey, ez, ax, ay, az);
    float mb = l1(ex, ey, ez, bxp, byp, bzp);
    float mc = l1(ex, ey, ez, cxp, cyp, czp);
    if (pc > 1 && mb < ma) {
        float t0 = ax; ax = bxp; bxp = t0; t0 = ay; ay = byp; byp = t0; t0 = az; az = bzp; bzp = t0;
        t0 = ma; ma = mb; mb = t0; int ti = ai; ai = bi; bi = ti;
    }
    if (pc > 2 && mc < ma) {
        float t0 = ax; ax = cxp; cxp = t0; t0 = ay; ay = cyp; cyp = t0; t0 = az; az = czp; czp = t0;
        t0 = ma; ma = mc; mc = t0; int ti = ai; ai = ci; ci = ti;
    }
    if (pc > 2 && mc < mb) {
        float t0 = bxp; bxp = cxp; cxp = t0; t0 = byp; byp = cyp; cyp = t0; t0 = bzp; bzp = czp; czp = t0;
        t0 = mb; mb = mc; mc = t0; int ti = bi; bi = ci; ci = ti;
    }
    uint32_t s1 = sub ^ (1u << ai), s2 = s1 ^ (1u << bi), s3 = s2 ^ (1u << ci);
    bool w1 = pc > 0 && ((mask >> s1) & 1u);
    bool w2 = pc > 1 && ((mask >> s2) & 1u);
    bool w3 = pc > 2 && ((mask >> s3) & 1u);
    int npush = (int)w1 + (int)w2 + (int)w3;
    if (s.sp + npush > CAP) return false;
    if (w3) stack[s.sp++] = make_uint4(link + VOXP_REC_UNITS * (uint32_t)__popc(mask & ((1u << s3) - 1u)),
                                       __float_as_uint(cxp), __float_as_uint(cyp), __float_as_uint(czp));
    if (w2) stack[s.sp++] = make_uint4(link + VOXP_REC_UNITS * (uint32_t)__popc(mask & ((1u << s2) - 1u)),
                                       __float_as_uint(bxp), __float_as_uint(byp), __float_as_uint(bzp));
    if (w1) stack[s.sp++] = make_uint4(link + VOXP_REC_UNITS * (uint32_t)__popc(mask & ((1u << s1) - 1u)),
                                       __float_as_uint(ax), __float_as_uint(ay), __float_as_uint(az));
    return true;
}

template <int CAP, bool COUNT>
__device__ __forceinline__ int ray_step(const DevTree &t, RaySearch &s, uint4 (&stack)[CAP], RayHit &hit,
                                        Counts &cnt)
{
    // Each node and each voxel is tested at most once per search, so more
    // steps than the tree holds means a damaged pool: stop with an error.
    if (++s.steps > t.max_steps) return STEP_ERROR;
    const uint4 *pool = t.pool;
    const float dx = s.dx, dy = s.dy, dz = s.dz;
    if (!in_range(s.scan ? (uint64_t)s.cur + s.vi : s.cur, s.scan ? 1u : VOXP_REC_UNITS, t.n_units, t.fault))
        return STEP_ERROR;
    uint4 u0 = ld16(pool + (s.scan ? s.cur + s.vi : s.cur));
    uint4 u1 = make_uint4(0u, 0u, 0u, 0u), u2 = make_uint4(0u, 0u, 0u, 0u);
    if (!s.scan) {
        u1 = ld16(pool + s.cur + 1);
        u2 = ld16(pool + s.cur + 2);
    }
    float lx = ubf(u0.x), ly = ubf(u0.y), lz = ubf(u0.z), hx, hy, hz;
    if (s.scan) {   // voxel box [dot, dot + vox_voxel] (search.c:53-54)
        hx = __fadd_rn(lx, t.vx); hy = __fadd_rn(ly, t.vy); hz = __fadd_rn(lz, t.vz);
        if (COUNT) cnt.voxels++;
    } else {
        hx = ubf(u0.w); hy = ubf(u1.x); hz = ubf(u1.y);
        if (COUNT) cnt.nodes++;
    }
    float ex, ey, ez;
    bool in = hit_box(lx, ly, lz, hx, hy, hz, s.ox, s.oy, s.oz, dx, dy, dz, ex, ey, ez);
    bool resume = false;

    if (s.scan) {
        // leaf loop body, search.c:55-78: nearest voxel by L1 distance from
        // the leaf's entry point, first one at distance 0 wins at once
        bool stop = false;
        if (in) {
            float dist = l1(s.ox, s.oy, s.oz, ex, ey, ez);
            if (dist == 0.0f) {
                s.bx = ex; s.by = ey; s.bz = ez; s.win = (int)s.vi; stop = true;
            } else if (dist < s.best) {
                s.best = dist; s.bx = ex; s.by = ey; s.bz = ez; s.win = (int)s.vi;
            }
        }
        s.vi++;
        if (stop || s.vi == s.vn) {
            if (s.win >= 0) {
                hit.x = s.bx; hit.y = s.by; hit.z = s.bz;
                hit.leaf = s.vid; hit.slot = (uint32_t)s.win; hit.rec = s.vrec;
                return STEP_HIT;
            }
            s.scan = false;
            resume = true;
        }
    } else if (!in) {
        resume = true;
    } else {
        uint32_t meta = u1.z, link = u1.w, kind = meta & 3u;
        if (kind == VOXP_KIND_DENSE) {                      // search.c:31-37
            hit.x = ex; hit.y = ey; hit.z = ez;
            hit.leaf = link; hit.slot = 0xFFu; hit.rec = s.cur;
            return STEP_HIT;
        }
        if (kind == VOXP_KIND_LEAF) {                       // search.c:39-50
            s.vn = meta >> 2;
            if (s.vn == 0) {
                resume = true;
            } else {
                s.scan = true; s.vrec = s.cur; s.vid = u2.x; s.cur = link; s.vi = 0;
                s.best = __int_as_float(0x7f800000); s.win = -1;
                s.ox = ex; s.oy = ey; s.oz = ez;
            }
        } else {                                            // inner node
            if (COUNT) cnt.inner++;
            float cx = ubf(u2.x), cy = ubf(u2.y), cz = ubf(u2.z);
            // geom.c:53-65 get_corrected_subspace_idx
            uint32_t sub = ((cx == ex) ? (dx < 0.0f) : (cx > ex))
                         | (((cy == ey) ? (dy < 0.0f) : (cy > ey)) << 1)
                         | (((cz == ez) ? (dz < 0.0f) : (cz > ez)) << 2);
            uint32_t mask = (meta >> 8) & 0xFFu;
            if (!push_crossings<CAP>(s, stack, ex, ey, ez, lx, ly, lz, hx, hy, hz, cx, cy, cz, sub, mask, link))
                return STEP_ERROR;
            if ((mask >> sub) & 1u) {                       // search.c:92-93
                s.cur = link + VOXP_REC_UNITS * (uint32_t)__popc(mask & ((1u << sub) - 1u));
                s.ox = ex; s.oy = ey; s.oz = ez;
            } else {
                resume = true;
            }
        }
    }
    if (resume) {
        if (s.sp == 0) return STEP_MISS;
        uint4 e = stack[--s.sp];
        s.cur = e.x;
        s.ox = ubf(e.y); s.oy = ubf(e.z); s.oz = ubf(e.w);
    }
    return STEP_MORE;
}

/* The whole search from the node whose record is at `start`.  Returns true
 * on a hit; `overflow` is set (and the search ends as a miss) on STEP_ERROR. */
template <int CAP, bool COUNT>
__device__ __forceinline__ bool trace_ray(const DevTree &t, uint32_t start,
                                          float ox0, float oy0, float oz0,
                                          float dx, float dy, float dz,
                                          RayHit &hit, Counts &cnt, bool &overflow)
{
    RaySearch s;
    uint4 stack[CAP];
    ray_begin(s, start, ox0, oy0, oz0, dx, dy, dz);
    for (;;) {
        int r = ray_step<CAP, COUNT>(t, s, stack, hit, cnt);
        if (r != STEP_MORE) {
            if (r == STEP_ERROR) overflow = true;
            return r == STEP_HIT;
        }
    }
}

/* geom.c:149-154 box_ball_interp with vox_sqr_metric (geom.c:133-139):
 * clamp the centre into the box, ((dx*dx + dy*dy) + dz*dz) < r*r. */
__device__ __forceinline__ bool ball_box(float lx, float ly, float lz, float hx, float hy, float hz,
                                         float cx, float cy, float cz, float rr)
{
    float fx = cx < lx ? lx : (cx > hx ? hx : cx);
    float fy = cy < ly ? ly : (cy > hy ? hy : cy);
    float fz = cz < lz ? lz : (cz > hz ? hz : cz);
    float ex = __fsub_rn(fx, cx), ey = __fsub_rn(fy, cy), ez = __fsub_rn(fz, cz);
    float s = __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
    return s < rr;
}

/* vox_tree_ball_collidep (search.c:155-183): any voxel box meeting the open
 * ball; children in octant order, first hit ends the search. */
template <int CAP, bool COUNT>
__device__ __forceinline__ bool trace_ball(const DevTree &t, float cx, float cy, float cz, float r,
                                           Counts &cnt, bool &overflow)
{
    if (t.root == VOXP_EMPTY) return false;
    uint32_t stack[CAP];
    int sp = 0;
    uint32_t cur = t.root;
    const uint4 *pool = t.pool;
    float rr = __fmul_rn(r, r);
    uint32_t steps = 0;
    for (;;) {
        if (++steps > t.max_steps) { overflow = true; return false; }   // damaged pool
        if (!in_range(cur, 2, t.n_units, t.fault)) { overflow = true; return false; }
        uint4 a = ld16(pool + cur);
        uint4 b = ld16(pool + cur + 1);
        if (COUNT) cnt.nodes++;
        if (ball_box(ubf(a.x), ubf(a.y), ubf(a.z), ubf(a.w), ubf(b.x), ubf(b.y), cx, cy, cz, rr)) {
            uint32_t kind = b.z & 3u, link = b.w;
            if (kind == VOXP_KIND_DENSE) return true;
            if (kind == VOXP_KIND_LEAF) {
                uint32_t n = b.z >> 2;
                if (!in_range(link, n, t.n_units, t.fault)) { overflow = true; return false; }
                for (uint32_t i = 0; i < n; i++) {
                    uint4 v = ld16(pool + link + i);
                    if (COUNT) cnt.voxels++;
                    float vx = ubf(v.x), vy = ubf(v.y), vz = ubf(v.z);
                    if (ball_box(vx, vy, vz, __fadd_rn(vx, t.vx), __fadd_rn(vy, t.vy),
                                 __fadd_rn(vz, t.vz), cx, cy, cz, rr))
                        return true;
                }
            } else {
                if (COUNT) cnt.inner++;
                uint32_t mask = (b.z >> 8) & 0xFFu;
                int k = __popc(mask);
                if (k > 0) {
                    if (sp + k - 1 > CAP) { overflow = true; return false; }
                    // children in octant order = consecutive records; push in
                    // reverse so octant order is the pop order.
                    for (int i = k - 1; i >= 1; i--) stack[sp++] = link + VOXP_REC_UNITS * (uint32_t)i;
                    cur = link;
                    continue;
                }
            }
        }
        if (sp == 0) return false;
        cur = stack[--sp];
    }
}

/* simple-camera.c:21-31 (+ vect-ops.c:7-15, :28-36) and doom-camera.c:24-57. */
__device__ __forceinline__ void screen2world(const vox_cuda_camera &cam, int sx, int sy,
                                             float &rx, float &ry, float &rz)
{
    float v0 = __fsub_rn(__fmul_rn(cam.mul, (float)sx), cam.xsub);
    float v2 = __fsub_rn(cam.ysub, __fmul_rn(cam.mul, (float)sy));
    if (cam.kind == VOX_CUDA_CAMERA_DOOM) {
        const float v1 = 1.0f;
        v2 = __fadd_rn(v2, cam.k);
        rx = __fsub_rn(__fmul_rn(v0, cam.cosphi), __fmul_rn(v1, cam.sinphi));
        ry = __fadd_rn(__fmul_rn(v1, cam.cosphi), __fmul_rn(v0, cam.sinphi));
        rz = v2;
        return;
    }
    const float v1 = 1.0f;
    float qw = cam.rotation[0], qi = cam.rotation[1], qj = cam.rotation[2], qk = cam.rotation[3];
    // t = 2 * (q.xyz x v)
    float t0 = __fsub_rn(__fmul_rn(qj, v2), __fmul_rn(qk, v1));
    float t1 = __fadd_rn(__fmul_rn(-qi, v2), __fmul_rn(qk, v0));
    float t2 = __fsub_rn(__fmul_rn(qi, v1), __fmul_rn(qj, v0));
    t0 = __fmul_rn(t0, 2.0f); t1 = __fmul_rn(t1, 2.0f); t2 = __fmul_rn(t2, 2.0f);
    // u = q.xyz x t
    float u0 = __fsub_rn(__fmul_rn(qj, t2), __fmul_rn(qk, t1));
    float u1 = __fadd_rn(__fmul_rn(-qi, t2), __fmul_rn(qk, t0));
    float u2 = __fsub_rn(__fmul_rn(qi, t1), __fmul_rn(qj, t0));
    rx = __fadd_rn(__fadd_rn(v0, __fmul_rn(qw, t0)), u0);
    ry = __fadd_rn(__fadd_rn(v1, __fmul_rn(qw, t1)), u1);
    rz = __fadd_rn(__fadd_rn(v2, __fmul_rn(qw, t2)), u2);
}

/* renderer.c:27-39 get_color without a light manager; SDL_MapRGB on an
 * ARGB8888 surface packs an opaque grey. */
__device__ __forceinline__ uint32_t texel_color(const uint8_t *__restrict__ tex, const DevTree &t,
                                                float x, float y, float z)
{
    int ix = abs(__float2int_rz(__fdiv_rn(x, t.vx))) & 31;
    int iy = abs(__float2int_rz(__fdiv_rn(y, t.vy))) & 31;
    int iz = abs(__float2int_rz(__fdiv_rn(z, t.vz))) & 31;
    uint32_t c = __ldg(tex + ix * 1024 + iy * 32 + iz);
    return 0xFF000000u | (c << 16) | (c << 8) | c;
}

/* Lights of a light manager on the device (layout: lights_internal.h).
 * nodes == nullptr: no bound lights, ambient only. */
struct DevLights {
    const float4 *nodes;     // 2 per M-tree node
    const float4 *spheres;   // 2 per light sphere
    float ar, ag, ab;        // ambient light
    uint32_t on;             // 0: draw without lights (grey texels)
    uint32_t n_nodes, n_spheres;
};

constexpr int LIGHT_STACK = 64;   // (children - 1) per level; the upload refuses deeper trees

/* geom.c:133-139 vox_sqr_metric: ((dx*dx + dy*dy) + dz*dz). */
__device__ __forceinline__ float sqr_dist(float ax, float ay, float az, float bx, float by, float bz)
{
    float x = __fsub_rn(ax, bx), y = __fsub_rn(ay, by), z = __fsub_rn(az, bz);
    return __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
}

/* lights.c:91-102 get_color_callback: the light of one sphere containing p. */
__device__ __forceinline__ void add_light(const float4 &sa, const float4 &sb, float px, float py, float pz,
                                          float &r, float &g, float &b)
{
    float dist = fminf(sb.w, __fsqrt_rn(sqr_dist(sa.x, sa.y, sa.z, px, py, pz)));
    float add = __fsub_rn(1.0f, __fdiv_rn(dist, sb.w));
    r = __fadd_rn(r, __fmul_rn(add, sb.x));
    g = __fadd_rn(g, __fmul_rn(add, sb.y));
    b = __fadd_rn(b, __fmul_rn(add, sb.z));
}

/* renderer.c:40-49 with lights.c:104-116 (vox_get_light) and
 * mtree.c:463-493 (vox_mtree_spheres_containing_f): ambient light plus the
 * spheres containing the hit, in the M-tree's depth-first order (a
 * one-sphere leaf whose bounding sphere holds the hit counts its sphere
 * without a second test), then min(light, 1) * texel per channel, truncated
 * to 8 bits.  `overflow` is set if the search stack would overflow. */
__device__ __forceinline__ uint32_t lit_color(const DevLights &L, uint32_t c, float px, float py, float pz,
                                              bool &overflow, uint32_t *fault)
{
    float r = L.ar, g = L.ag, b = L.ab;
    if (L.nodes) {
        uint32_t stack[LIGHT_STACK];
        int sp = 0;
        uint32_t cur = 0;
        for (;;) {
            if (!in_range(cur, 1, L.n_nodes, fault)) { overflow = true; break; }
            float4 na = L.nodes[2 * cur];
            float4 nb = L.nodes[2 * cur + 1];
            uint32_t leaf = __float_as_uint(nb.x), num = __float_as_uint(nb.y), first = __float_as_uint(nb.z);
            bool next_from_stack = true;
            if (sqr_dist(na.x, na.y, na.z, px, py, pz) < na.w) {
                if (leaf) {
                    if (!in_range(first, num, L.n_spheres, fault)) { overflow = true; break; }
                    if (num == 1) {
                        add_light(L.spheres[2 * first], L.spheres[2 * first + 1], px, py, pz, r, g, b);
                    } else {
                        for (uint32_t i = 0; i < num; i++) {
                            float4 sa = L.spheres[2 * (first + i)];
                            if (sqr_dist(sa.x, sa.y, sa.z, px, py, pz) < sa.w)
                                add_light(sa, L.spheres[2 * (first + i) + 1], px, py, pz, r, g, b);
                        }
                    }
                } else if (num > 0) {
                    if (sp + (int)num - 1 > LIGHT_STACK) { overflow = true; break; }
                    for (uint32_t i = num - 1; i >= 1; i--) stack[sp++] = first + i;
                    cur = first;
                    next_from_stack = false;
                }
            }
            if (next_from_stack) {
                if (sp == 0) break;
                cur = stack[--sp];
            }
        }
    }
    uint32_t R = __float2uint_rz(__fmul_rn(fminf(r, 1.0f), (float)c));
    uint32_t G = __float2uint_rz(__fmul_rn(fminf(g, 1.0f), (float)c));
    uint32_t B = __float2uint_rz(__fmul_rn(fminf(b, 1.0f), (float)c));
    return 0xFF000000u | ((R & 0xFFu) << 16) | ((G & 0xFFu) << 8) | (B & 0xFFu);
}

/* renderer.c:27-52 get_color: the texel of the hit point, grey without a
 * light manager (SDL_MapRGB on ARGB8888), lit with one. */
__device__ __forceinline__ uint32_t hit_color(const uint8_t *__restrict__ tex, const DevTree &t, const DevLights &L,
                                              float x, float y, float z, bool &overflow)
{
    int ix = abs(__float2int_rz(__fdiv_rn(x, t.vx))) & 31;
    int iy = abs(__float2int_rz(__fdiv_rn(y, t.vy))) & 31;
    int iz = abs(__float2int_rz(__fdiv_rn(z, t.vz))) & 31;
    uint32_t c = __ldg(tex + ix * 1024 + iy * 32 + iz);
    if (!L.on) return 0xFF000000u | (c << 16) | (c << 8) | c;
    return lit_color(L, c, x, y, z, overflow, t.fault);
}

}  // namespace vox

#endif
