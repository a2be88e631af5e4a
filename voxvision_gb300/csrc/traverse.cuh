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
 * Recursion becomes an explicit per-thread stack of tasks {record offset,
 * ray origin}.  vox_ray_tree_intersection (search.c:8-153) explores, for an
 * inner node, the child holding the entry point first and then -- only if
 * that found nothing -- the children behind each dividing plane the ray
 * crosses, nearest plane first.  The second half is deferred as a
 * "continuation" task {record offset | CONT | first octant << 28, entry
 * point}; popping it computes the plane crossings and pushes the children in
 * visiting order.  The first hit ends the search, exactly as the recursion
 * returns on its first non-NULL result.
 */
#ifndef VOX_TRAVERSE_CUH
#define VOX_TRAVERSE_CUH

#include <cstdint>
#include <cuda_runtime.h>

#include "pool_layout.h"
#include "../../include/voxtrees_cuda.h"

namespace vox {

constexpr uint32_t CONT_BIT = 0x80000000u;

struct DevTree {
    const uint4 *pool;
    const uint32_t *rec_of_id;   // pre-order id -> record offset
    uint32_t root;               // record offset of the root, VOXP_EMPTY if none
    uint32_t n_nodes;
    float vx, vy, vz;            // vox_voxel at upload time
};

struct Counts {
    uint32_t nodes, inner, voxels;
};

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

/* geom.c:101-123 hit_plane_within_box for axis p. */
__device__ __forceinline__ bool hit_plane(int p, float ox, float oy, float oz, float dx, float dy, float dz,
                                          float cp, float lx, float ly, float lz, float hx, float hy, float hz,
                                          float &rx, float &ry, float &rz)
{
    float op = p == 0 ? ox : (p == 1 ? oy : oz);
    float dp = p == 0 ? dx : (p == 1 ? dy : dz);
    float k = __fsub_rn(cp, op);
    if (k == 0.0f || ((dp < 0.0f) != (k < 0.0f))) return false;
    k = __fdiv_rn(k, dp);
    rx = __fadd_rn(ox, __fmul_rn(k, dx));
    if (rx < lx || rx > hx) return false;
    ry = __fadd_rn(oy, __fmul_rn(k, dy));
    if (ry < ly || ry > hy) return false;
    rz = __fadd_rn(oz, __fmul_rn(k, dz));
    if (rz < lz || rz > hz) return false;
    return true;
}

struct RayHit {
    float x, y, z;
    uint32_t leaf;    // pre-order id
    uint32_t slot;    // winning voxel, 0xFF for dense
    uint32_t rec;     // record offset of the leaf
};

/* vox_ray_tree_intersection (search.c:8-153) from the node whose record is at
 * `start`.  Returns true on a hit.  `overflow` is set (and the search ends
 * as a miss) if the stack would exceed CAP entries, which the upload-time
 * depth check rules out. */
template <int CAP, bool COUNT>
__device__ __forceinline__ bool trace_ray(const DevTree &t, uint32_t start,
                                          float ox0, float oy0, float oz0,
                                          float dx, float dy, float dz,
                                          RayHit &hit, Counts &cnt, bool &overflow)
{
    uint4 stack[CAP];
    int sp = 0;
    uint32_t cur = start;
    float ox = ox0, oy = oy0, oz = oz0;
    const uint4 *pool = t.pool;

    for (;;) {
        if (!(cur & CONT_BIT)) {
            // ---- visit a node: search.c:22-97
            uint4 a = ld16(pool + cur);
            uint4 b = ld16(pool + cur + 1);
            if (COUNT) cnt.nodes++;
            float lx = ubf(a.x), ly = ubf(a.y), lz = ubf(a.z);
            float hx = ubf(a.w), hy = ubf(b.x), hz = ubf(b.y);
            uint32_t meta = b.z, link = b.w;
            float ex, ey, ez;
            if (hit_box(lx, ly, lz, hx, hy, hz, ox, oy, oz, dx, dy, dz, ex, ey, ez)) {
                uint32_t kind = meta & 3u;
                if (kind == VOXP_KIND_DENSE) {              // :31-37
                    hit.x = ex; hit.y = ey; hit.z = ez;
                    hit.leaf = link; hit.slot = 0xFFu; hit.rec = cur;
                    return true;
                }
                if (kind == VOXP_KIND_LEAF) {               // :39-81
                    uint32_t n = meta >> 2;
                    float best = __int_as_float(0x7f800000);
                    int win = -1;
                    float bx = 0.f, by = 0.f, bz = 0.f;
                    for (uint32_t i = 0; i < n; i++) {
                        uint4 v = ld16(pool + link + i);
                        if (COUNT) cnt.voxels++;
                        float vx = ubf(v.x), vy = ubf(v.y), vz = ubf(v.z);
                        float fx, fy, fz;
                        if (hit_box(vx, vy, vz, __fadd_rn(vx, t.vx), __fadd_rn(vy, t.vy),
                                    __fadd_rn(vz, t.vz), ex, ey, ez, dx, dy, dz, fx, fy, fz)) {
                            float dist = l1(ex, ey, ez, fx, fy, fz);
                            if (dist == 0.0f) {
                                bx = fx; by = fy; bz = fz; win = (int)i;
                                break;
                            }
                            if (dist < best) {
                                best = dist;
                                bx = fx; by = fy; bz = fz; win = (int)i;
                            }
                        }
                    }
                    if (win >= 0) {
                        hit.x = bx; hit.y = by; hit.z = bz;
                        hit.leaf = ld16(pool + link - 1).x;
                        hit.slot = (uint32_t)win; hit.rec = cur;
                        return true;
                    }
                } else {                                    // inner, :84-97
                    if (COUNT) cnt.inner++;
                    uint4 c = ld16(pool + link);
                    float cx = ubf(c.x), cy = ubf(c.y), cz = ubf(c.z);
                    // geom.c:53-65 get_corrected_subspace_idx
                    uint32_t sub = ((cx == ex) ? (dx < 0.0f) : (cx > ex))
                                 | (((cy == ey) ? (dy < 0.0f) : (cy > ey)) << 1)
                                 | (((cz == ez) ? (dz < 0.0f) : (cz > ez)) << 2);
                    uint32_t mask = (meta >> 8) & 0xFFu;
                    if (sp >= CAP) { overflow = true; return false; }
                    stack[sp++] = make_uint4(cur | CONT_BIT | (sub << VOXP_OFF_BITS),
                                             __float_as_uint(ex), __float_as_uint(ey),
                                             __float_as_uint(ez));
                    if ((mask >> sub) & 1u) {
                        cur = link + 1u + 2u * (uint32_t)__popc(mask & ((1u << sub) - 1u));
                        ox = ex; oy = ey; oz = ez;
                        continue;
                    }
                }
            }
        } else {
            // ---- the entry octant found nothing: planes, search.c:105-148
            uint32_t node = cur & VOXP_OFF_MASK;
            uint32_t sub = (cur >> VOXP_OFF_BITS) & 7u;
            uint4 a = ld16(pool + node);
            uint4 b = ld16(pool + node + 1);
            uint32_t link = b.w, mask = (b.z >> 8) & 0xFFu;
            uint4 c = ld16(pool + link);
            float lx = ubf(a.x), ly = ubf(a.y), lz = ubf(a.z);
            float hx = ubf(a.w), hy = ubf(b.x), hz = ubf(b.y);
            float px[3], py[3], pz[3];
            int pidx[3];
            int pc = 0;
#pragma unroll
            for (int p = 0; p < 3; p++) {
                float cp = p == 0 ? ubf(c.x) : (p == 1 ? ubf(c.y) : ubf(c.z));
                float rx, ry, rz;
                if (hit_plane(p, ox, oy, oz, dx, dy, dz, cp, lx, ly, lz, hx, hy, hz, rx, ry, rz)) {
                    px[pc] = rx; py[pc] = ry; pz[pc] = rz; pidx[pc] = p; pc++;
                }
            }
            // The reference's in-place selection sort (search.c:115-134): strict
            // '<' and immediate swaps, reproduced exactly including its order
            // among equal distances.
            float m[3];
#pragma unroll
            for (int i = 0; i < 3; i++) m[i] = i < pc ? l1(ox, oy, oz, px[i], py[i], pz[i]) : 0.0f;
#pragma unroll
            for (int i = 0; i < 2; i++) {
#pragma unroll
                for (int j = i + 1; j < 3; j++) {
                    if (j < pc && m[j] < m[i]) {
                        float tx = px[i], ty = py[i], tz = pz[i], tm = m[i];
                        int ti = pidx[i];
                        px[i] = px[j]; py[i] = py[j]; pz[i] = pz[j]; m[i] = m[j]; pidx[i] = pidx[j];
                        px[j] = tx; py[j] = ty; pz[j] = tz; m[j] = tm; pidx[j] = ti;
                    }
                }
            }
            // Octants visited after each crossing (search.c:137) and their
            // records; NULL children are skipped (they return NULL at once).
            uint32_t recs[3];
            int nt = 0;
            uint32_t s = sub;
            float qx[3], qy[3], qz[3];
#pragma unroll
            for (int i = 0; i < 3; i++) {
                if (i < pc) {
                    s ^= 1u << pidx[i];
                    if ((mask >> s) & 1u) {
                        recs[nt] = link + 1u + 2u * (uint32_t)__popc(mask & ((1u << s) - 1u));
                        qx[nt] = px[i]; qy[nt] = py[i]; qz[nt] = pz[i];
                        nt++;
                    }
                }
            }
            if (nt > 0) {
                if (sp + nt - 1 > CAP) { overflow = true; return false; }
#pragma unroll
                for (int i = 2; i >= 1; i--) {
                    if (i < nt)
                        stack[sp++] = make_uint4(recs[i], __float_as_uint(qx[i]),
                                                 __float_as_uint(qy[i]), __float_as_uint(qz[i]));
                }
                cur = recs[0];
                ox = qx[0]; oy = qy[0]; oz = qz[0];
                continue;
            }
        }
        // ---- nothing found below this task: resume the deferred work
        if (sp == 0) return false;
        uint4 e = stack[--sp];
        cur = e.x;
        ox = ubf(e.y); oy = ubf(e.z); oz = ubf(e.w);
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
    for (;;) {
        uint4 a = ld16(pool + cur);
        uint4 b = ld16(pool + cur + 1);
        if (COUNT) cnt.nodes++;
        if (ball_box(ubf(a.x), ubf(a.y), ubf(a.z), ubf(a.w), ubf(b.x), ubf(b.y), cx, cy, cz, rr)) {
            uint32_t kind = b.z & 3u, link = b.w;
            if (kind == VOXP_KIND_DENSE) return true;
            if (kind == VOXP_KIND_LEAF) {
                uint32_t n = b.z >> 2;
                for (uint32_t i = 0; i < n; i++) {
                    uint4 v = ld16(pool + link + i);
                    if (COUNT) cnt.voxels++;
                    float vx = ubf(v.x), vy = ubf(v.y), vz = ubf(v.z);
                    if (ball_box(vx, vy, vz, __fadd_rn(vx, t.vx), __fadd_rn(vy, t.vy),
                                 __fadd_rn(vz, t.vz), cx, cy, cz, rr))
                        return true;
                }
            } else {
                uint32_t mask = (b.z >> 8) & 0xFFu;
                int k = __popc(mask);
                if (k > 0) {
                    if (sp + k - 1 > CAP) { overflow = true; return false; }
                    // children in octant order = consecutive records; push in
                    // reverse so octant order is the pop order.
                    for (int i = k - 1; i >= 1; i--) stack[sp++] = link + 1u + 2u * (uint32_t)i;
                    cur = link + 1u;
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

}  // namespace vox

#endif
