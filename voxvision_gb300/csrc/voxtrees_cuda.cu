/*
 * voxtrees_cuda.cu -- kernels and the C ABI of libvoxtrees_cuda
 * (declared in include/voxtrees_cuda.h).
 *
 * Kernels (one thread per query, traversal in traverse.cuh):
 *   ray_kernel     batched vox_ray_tree_intersection, optional per-ray roots
 *   ball_kernel    batched vox_tree_ball_collidep
 *   render_kernel  vox_render BEST: camera ray, search and colour fused; a
 *                  warp covers an 8x4 pixel tile, a block 16x8 pixels, so the
 *                  rays of a warp are neighbours and walk the same nodes.
 * Each has a counting twin (COUNT=true) that only tallies the work.
 *
 * The stack capacity is a template parameter picked from the tree depth at
 * upload time, so a kernel never needs more stack than it has.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "flatten.h"
#include "lights_internal.h"
#include "internal.h"
#include "pool_layout.h"
#include "traverse.cuh"
#include "../../include/voxtrees_cuda.h"
#include "abi_guard.h"

#define EXPORT extern "C" __attribute__((visibility("default")))

using vox::Counts;
using vox::centre_out;
using vox::DevTree;
using vox::RayHit;
using vox::FramePlan;
using vox::FrameMemo;

namespace {

std::atomic<uint64_t> g_launches{0};

__device__ __forceinline__ void add_counts(unsigned long long *counts, const Counts &c)
{
    unsigned long long n = c.nodes, i = c.inner, v = c.voxels;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        n += __shfl_down_sync(0xffffffffu, n, o);
        i += __shfl_down_sync(0xffffffffu, i, o);
        v += __shfl_down_sync(0xffffffffu, v, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counts + 0, n);
        atomicAdd(counts + 1, i);
        atomicAdd(counts + 2, v);
    }
}

template <int CAP, bool COUNT>
__global__ void __launch_bounds__(256) ray_kernel(DevTree t, const float *__restrict__ o,
                                                  const float *__restrict__ d,
                                                  const uint32_t *__restrict__ roots, size_t n,
                                                  uint32_t *__restrict__ leaf, uint8_t *__restrict__ slot,
                                                  float *__restrict__ pts,
                                                  unsigned long long *__restrict__ counts,
                                                  uint32_t *__restrict__ status,
                                                  const uint32_t *__restrict__ order)
{
    size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    Counts c{0, 0, 0};
    bool overflow = false;
    if (j < n) {
        size_t i = order ? order[j] : j;   // the j-th ray traced (raysort.cu)
        uint32_t start = t.root;
        if (roots) {
            uint32_t id = roots[i];
            start = (id < t.n_nodes) ? t.rec_of_id[id] : (id == VOX_CUDA_MISS ? t.root : VOXP_EMPTY);
        }
        RayHit h;
        bool hit = false;
        if (start != VOXP_EMPTY)
            hit = vox::trace_ray<CAP, COUNT>(t, start, o[3 * i], o[3 * i + 1], o[3 * i + 2],
                                             d[3 * i], d[3 * i + 1], d[3 * i + 2], h, c, overflow);
        if (!COUNT) {
            leaf[i] = hit ? h.leaf : VOX_CUDA_MISS;
            if (slot) slot[i] = hit ? (uint8_t)h.slot : (uint8_t)0xFF;
            if (hit && pts) {
                pts[3 * i] = h.x; pts[3 * i + 1] = h.y; pts[3 * i + 2] = h.z;
            }
        }
        if (overflow) atomicOr(status, 1u);
    }
    if (COUNT) add_counts(counts, c);
}

template <int CAP, bool COUNT>
__global__ void __launch_bounds__(256) ball_kernel(DevTree t, const float *__restrict__ ctr,
                                                   const float *__restrict__ rad, size_t n,
                                                   uint8_t *__restrict__ hit,
                                                   unsigned long long *__restrict__ counts,
                                                   uint32_t *__restrict__ status,
                                                   const uint32_t *__restrict__ order)
{
    size_t j = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    Counts c{0, 0, 0};
    bool overflow = false;
    if (j < n) {
        size_t i = order ? order[j] : j;   // the j-th ball searched (raysort.cu)
        bool h = vox::trace_ball<4 * CAP, COUNT>(t, ctr[3 * i], ctr[3 * i + 1], ctr[3 * i + 2], rad[i],
                                                 c, overflow);
        if (!COUNT) hit[i] = h ? 1 : 0;
        if (overflow) atomicOr(status, 1u);
    }
    if (COUNT) add_counts(counts, c);
}

// vox_render BEST (renderer.c:200-319, branch :308): camera ray, search and
// colour fused, one thread per pixel.  A warp covers an 8x4 pixel tile, a
// block 16x8, so the rays of a warp are neighbours and walk the same nodes.
//
// Only the blocks of the screen rectangle that the tree's bounding box can
// project into are traced (FramePlan, planned on the host); they are issued
// outward from where the tree's centre projects, so the rays that walk the
// tree longest start first.  The blocks after them clear the rest of the
// frame: those pixels are misses.
//
// Overlap with the previous kernel of the stream (PDL): the kernel is
// launched with programmatic stream serialisation and lets its own successor
// start as soon as all its blocks are running (launch_dependents).  Before
// griddepcontrol.wait it reads only the tree's pool (written once, at upload,
// before the upload returns) and its parameters; the texture, the frame, the
// status word and the counters are touched only after the wait, which
// returns once the previous kernel has completed and its memory is visible.
// So the traversal of this frame runs in the tail of the previous one while
// every read and write of stream-ordered memory keeps the stream's order.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// A clearing block of a frame launch (block index ntiles and up): the
// clearing rectangle of the plan outside the traced one, rows dealt to the
// block's warps; a warp's lanes store 16 bytes each when the frame is 16-byte
// aligned (row starts and every bound then are: w is a multiple of 16, the
// rectangles' x bounds of 8 or w).
__device__ __forceinline__ void clear_outside(const FramePlan &p, uint32_t w, uint32_t h, uint32_t *argb,
                                              uint32_t warp, uint32_t lane)
{
    const bool vec = (reinterpret_cast<uintptr_t>(argb) & 15u) == 0;
    const uint32_t nw = (gridDim.x - p.ntiles) * 4u;
    for (uint32_t y = p.cy0 + (blockIdx.x - p.ntiles) * 4u + warp; y < p.cy1; y += nw) {
        uint32_t *row = argb + (size_t)y * w;
        uint32_t a0 = p.cx0, b0 = p.cx1, a1 = 0, b1 = 0;  // the row's part of the clearing rectangle,
        if (y >= p.y0 && y < p.y1) {                       // or its two margins beside the traced one
            b0 = min(p.cx1, max(p.cx0, p.x0));
            a1 = max(p.cx0, min(p.cx1, p.x1));
            b1 = p.cx1;
        }
        if (vec) {
            uint4 *r4 = reinterpret_cast<uint4 *>(row);
            for (uint32_t i = a0 / 4 + lane; i < b0 / 4; i += 32) r4[i] = make_uint4(0u, 0u, 0u, 0u);
            for (uint32_t i = a1 / 4 + lane; i < b1 / 4; i += 32) r4[i] = make_uint4(0u, 0u, 0u, 0u);
        } else {
            for (uint32_t i = a0 + lane; i < b0; i += 32) row[i] = 0u;
            for (uint32_t i = a1 + lane; i < b1; i += 32) row[i] = 0u;
        }
    }
}

template <int CAP, bool COUNT, int MINB, bool LIT>
__global__ void __launch_bounds__(128, MINB) render_kernel(DevTree t, vox_cuda_camera cam, uint32_t w, uint32_t h,
                                                     FramePlan p, const uint8_t *__restrict__ tex,
                                                     uint32_t *__restrict__ argb,
                                                     unsigned long long *__restrict__ counts,
                                                     uint32_t *__restrict__ status, vox::DevLights lights)
{
    pdl_launch_dependents();
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (blockIdx.x >= p.ntiles) {
        pdl_wait();
        if (!COUNT) clear_outside(p, w, h, argb, warp, lane);
        return;
    }
    uint32_t by = centre_out(blockIdx.x / p.ntx, p.cty, p.nty);
    uint32_t bx = centre_out(blockIdx.x % p.ntx, p.ctx, p.ntx);
    uint32_t px = p.x0 + bx * TILE_W + (warp & 1) * 8 + (lane & 7);
    uint32_t py = p.y0 + by * TILE_H + (warp >> 1) * 4 + (lane >> 3);
    Counts c{0, 0, 0};
    bool overflow = false, hit = false, mine = px < p.x1 && py < p.y1;
    RayHit hh;
    if (mine) {
        float dx, dy, dz;
        vox::screen2world(cam, (int)px, (int)py, dx, dy, dz);
        if (t.root != VOXP_EMPTY)
            hit = vox::trace_ray<CAP, COUNT>(t, t.root, cam.position[0], cam.position[1], cam.position[2],
                                             dx, dy, dz, hh, c, overflow);
    }
    pdl_wait();
    if (mine) {
        if (!COUNT) {
            uint32_t colour = 0u;
            if (hit) colour = LIT ? vox::hit_color(tex, t, lights, hh.x, hh.y, hh.z, overflow)
                                  : vox::texel_color(tex, t, hh.x, hh.y, hh.z);
            argb[(size_t)py * w + px] = colour;
        }
        if (overflow) atomicOr(status, 1u);
    }
    if (COUNT) add_counts(counts, c);
}

// vox_render in FAST / ADAPTIVE quality (renderer.c:215-318): each 4x4
// square's 16 pixels in the reference's Z-order, reusing the previous pixel's
// leaf as the search root (FAST) and choosing the mode per square from the
// two corner rays (ADAPTIVE), with optional ray merging.
__device__ __forceinline__ float sqr3(float ax, float ay, float az, float bx, float by, float bz)
{
    float x = __fsub_rn(ax, bx), y = __fsub_rn(ay, by), z = __fsub_rn(az, bz);
    return __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
}

// The direction of pixel (x, y): the camera's screen2world, or with RAYS the
// pixel's entry of a ray buffer (3 floats a pixel, rows of w pixels) that the
// host filled through a camera class the device cannot compute.
template <bool RAYS>
__device__ __forceinline__ void pixel_dir(const vox_cuda_camera &cam, const float *__restrict__ rays, uint32_t w,
                                          int x, int y, float &dx, float &dy, float &dz)
{
    if (RAYS) {
        const float *r = rays + 3 * ((size_t)y * w + (uint32_t)x);
        dx = r[0]; dy = r[1]; dz = r[2];
    } else {
        vox::screen2world(cam, x, y, dx, dy, dz);
    }
}

// Register bound of render_squares_kernel: none by default (72 registers, 7
// blocks of 128 threads per SM).  Bounds of 8 and 9 blocks (64 and 56
// registers, with spills) drew the 1080p orbit's FAST and ADAPTIVE frames 1-3%
// slower.
#ifdef SQUARES_MIN_BLOCKS
#define SQUARES_BOUNDS __launch_bounds__(128, SQUARES_MIN_BLOCKS)
#else
#define SQUARES_BOUNDS __launch_bounds__(128)
#endif

// FAST and ADAPTIVE frames, and with a ray buffer frames of every quality,
// in one launch.  In renderer.c a pixel's leaf is either the previous
// pixel's leaf, when the ray meets a voxel there (the search from the leaf,
// :297), or what the search from the root finds for the pixel's own ray
// (:299, and every corner and BEST pixel); the second never depends on the
// square's earlier pixels.  So each half-warp holds one 4x4 square, a pixel
// a lane (a warp is two squares side by side, 8x4 pixels, the BEST kernel's
// warp tile): every lane first makes the root search of its own ray, then
// the lanes still to be drawn make, at once, the search from the leaf the
// square's walk currently holds.  The walk itself -- the reference's 16
// pixels in its order, with its choices of mode, merging and leaf -- runs on
// every lane of the square alike over ballots of those results, and
// wherever it changes to a leaf the round's searches were not made from, a
// new round makes them for the pixels after it.  A square takes one round
// per change of leaf, and the leaf rarely changes within a square.  The
// results are the reference's by construction: the same searches of the
// same rays, the same choices between them; searches made for pixels the
// walk then reaches another way are dropped.
template <int CAP, bool RAYS>
__global__ void SQUARES_BOUNDS render_squares_kernel(DevTree t, vox_cuda_camera cam, uint32_t w, uint32_t h,
                                                     FramePlan fp, unsigned int quality,
                                                     const uint8_t *__restrict__ tex, uint32_t *__restrict__ argb,
                                                     uint32_t *__restrict__ status, vox::DevLights lights,
                                                     const float *__restrict__ rays)
{
    // renderer.c:23-25 rendering order {0, 1, 4, 5, 2, 3, 6, 7, 8, 9, 12, 13, 10, 11, 14, 15}, a nibble
    // each; the permutation is its own inverse, so it also maps a pixel to its place in the order
    constexpr uint64_t ORDER = 0xFEBADC9876325410ull;
    constexpr unsigned FULL = 0xFFFFFFFFu;
    pdl_launch_dependents();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, p = lane & 15;
    if (blockIdx.x >= fp.ntiles) {                  // the frame outside the rectangle: misses
        pdl_wait();
        clear_outside(fp, w, h, argb, warp, lane);
        return;
    }
    if (RAYS) pdl_wait();                           // the ray buffer is stream-ordered memory
    const int ip = (int)((ORDER >> (4 * p)) & 15u);                        // this pixel's place in the order
    const uint32_t by = centre_out(blockIdx.x / fp.ntx, fp.cty, fp.nty);
    const uint32_t bx = centre_out(blockIdx.x % fp.ntx, fp.ctx, fp.ntx);
    const uint32_t xstart = fp.x0 + bx * TILE_W + (warp & 1) * 8 + (lane >> 4) * 4;
    const uint32_t ystart = fp.y0 + by * TILE_H + (warp >> 1) * 4;
    const bool valid = xstart < fp.x1 && ystart < fp.y1;                    // whole squares: all 16 lanes alike
    const int px = (int)xstart + (p & 3), py = (int)ystart + (p >> 2);
    const float ox = cam.position[0], oy = cam.position[1], oz = cam.position[2];
    const int rnd_mode = quality & VOX_CUDA_QUALITY_MODE_MASK;
    const int merge_mode = quality & VOX_CUDA_QUALITY_RM_MASK;
    Counts c{0, 0, 0};
    bool overflow = false;

    // the root search of this pixel's ray
    float dx = 0.f, dy = 0.f, dz = 0.f;
    uint32_t rrec = VOXP_EMPTY;
    float rx = 0.f, ry = 0.f, rz = 0.f;
    if (valid) {
        pixel_dir<RAYS>(cam, rays, w, px, py, dx, dy, dz);
        RayHit hh;
        if (t.root != VOXP_EMPTY && vox::trace_ray<CAP, false>(t, t.root, ox, oy, oz, dx, dy, dz, hh, c, overflow)) {
            rrec = hh.rec;
            rx = hh.x; ry = hh.y; rz = hh.z;
        }
    }

    // the square's mode (renderer.c:240-282), alike on its 16 lanes
    int mode = rnd_mode, istart = 0, iend = 16;
    bool bmerge = false, have = false;       // `leaf != NULL` of renderer.c
    uint32_t leaf = VOXP_EMPTY;
    const uint32_t c1 = __shfl_sync(FULL, rrec, 0, 16), c2 = __shfl_sync(FULL, rrec, 15, 16);
    const float ix = __shfl_sync(FULL, rx, 0, 16), iy = __shfl_sync(FULL, ry, 0, 16), iz = __shfl_sync(FULL, rz, 0, 16);
    const float jx = __shfl_sync(FULL, rx, 15, 16), jy = __shfl_sync(FULL, ry, 15, 16), jz = __shfl_sync(FULL, rz, 15, 16);
    const float d1x = __shfl_sync(FULL, dx, 0, 16), d1y = __shfl_sync(FULL, dy, 0, 16), d1z = __shfl_sync(FULL, dz, 0, 16);
    const float d2x = __shfl_sync(FULL, dx, 15, 16), d2y = __shfl_sync(FULL, dy, 15, 16), d2z = __shfl_sync(FULL, dz, 15, 16);
    bool res_have = false, res_merge = false;    // this pixel: drawn from a hit / copied from the previous pixel
    float qx = rx, qy = ry, qz = rz;              // and its intersection point
    if (rnd_mode == VOX_CUDA_QUALITY_ADAPTIVE) {
        bmerge = (merge_mode == VOX_CUDA_QUALITY_RAY_MERGE);
        istart = 1;
        mode = VOX_CUDA_QUALITY_FAST;
        have = c1 != VOXP_EMPTY;
        leaf = c1;
        if (p == 0) res_have = have;                                        // corner 1, drawn now
        if (have) {
            iend = 15;
            if (c2 != VOXP_EMPTY) {
                if (p == 15) res_have = true;                               // corner 2, drawn now
                float d1 = sqr3(ix, iy, iz, ox, oy, oz);
                float d2 = sqr3(d1x, d1y, d1z, 0.f, 0.f, 0.f);
                float criteria = __fmul_rn(__fdiv_rn(d1, d2), sqr3(d1x, d1y, d1z, d2x, d2y, d2z));
                float dist = sqr3(ix, iy, iz, jx, jy, jz);
                if ((double)__fdiv_rn(dist, criteria) > 1.69)               // LENGTH_THRESHOLD, renderer.c:197
                    mode = VOX_CUDA_QUALITY_BEST;
                if (d1 > 22500.0f)                                          // MAX_DIST^2, renderer.c:198
                    bmerge = (mode == VOX_CUDA_QUALITY_FAST && merge_mode == VOX_CUDA_QUALITY_RAY_MERGE_ACCURATE)
                                 ? true : bmerge;
                else
                    bmerge = false;
            }
        }
    }

    // the walk (renderer.c:286-315) in rounds of searches from one leaf.  The
    // walk's decisions need, per pixel, only whether its search from the
    // round's leaf met a voxel, whether its root search did, and whether that
    // found the round's leaf: three ballots a round, after which every lane
    // of the square walks the same 16-bit masks; a pixel's point is its own
    // lane's (from the leaf or from the root, as the walk decides).
    const int seg = lane & 16;                    // first lane of this square
    const unsigned nonempty = (__ballot_sync(FULL, rrec != VOXP_EMPTY) >> seg) & 0xFFFFu;
    bool from_leaf = false;                       // this pixel's point is its search from the leaf
    int pos = istart;                             // the next place in the order still to be walked
    for (;;) {
        const bool pending = valid && pos < iend;
        if (!__any_sync(FULL, pending)) break;
        const bool searched = mode == VOX_CUDA_QUALITY_FAST && have;      // this round's searches are from `leaf`
        bool shit = false;
        float sx = 0.f, sy = 0.f, sz = 0.f;
        if (pending && searched && ip >= pos && ip < iend && !(bmerge && (ip & 1))) {
            RayHit hh;
            if (vox::trace_ray<CAP, false>(t, leaf, ox, oy, oz, dx, dy, dz, hh, c, overflow)) {
                shit = true;
                sx = hh.x; sy = hh.y; sz = hh.z;
            }
        }
        const unsigned hits = (__ballot_sync(FULL, shit) >> seg) & 0xFFFFu;
        const unsigned same = (__ballot_sync(FULL, rrec == leaf) >> seg) & 0xFFFFu;
        int stop = iend, next = -1;                 // where the round ends, and the pixel whose leaf comes next
        for (int i = pos; pending && i < stop; i++) {
            const int pi = (int)((ORDER >> (4 * i)) & 15u);
            const unsigned bit = 1u << pi;
            const bool merge = bmerge && (i & 1);
            bool leafed = false;
            if (!merge) {
                if (mode == VOX_CUDA_QUALITY_FAST && have && (hits & bit)) {   // the search from the leaf met a voxel
                    leafed = true;
                } else {                                                       // ... else the pixel's root result
                    have = (nonempty & bit) != 0;
                    // later pixels search from this leaf: if this round searched from another, a new round
                    if (have && mode == VOX_CUDA_QUALITY_FAST && !(searched && (same & bit))) {
                        stop = i + 1;
                        next = pi;
                    }
                }
            }
            if (p == pi) {
                res_have = have;
                res_merge = merge;
                from_leaf = leafed;
            }
        }
        if (from_leaf && ip >= pos && ip < stop) {
            qx = sx; qy = sy; qz = sz;
        }
        // the leaf the walk holds now: unchanged, or the root result of pixel `next`
        const uint32_t nl = __shfl_sync(FULL, rrec, next < 0 ? 0 : next, 16);
        if (next >= 0) leaf = nl;
        pos = stop;
    }

    // colours: a merged pixel takes the previous pixel's (renderer.c:309);
    // the texture, the lights and the frame are stream-ordered memory
    pdl_wait();
    uint32_t color = 0u;
    if (valid && res_have && !res_merge) color = vox::hit_color(tex, t, lights, qx, qy, qz, overflow);
    const int prev = ip > 0 ? (int)((ORDER >> (4 * (ip - 1))) & 15u) : 0;
    const uint32_t pcol = __shfl_sync(FULL, color, prev, 16);
    if (res_merge) color = res_have ? pcol : 0u;
    if (valid) argb[(size_t)py * w + px] = color;
    if (overflow) atomicOr(status, 1u);
}

// ---------------------------------------------------------------- launchers

// Batches of at least this many rays are traced in coherent order (raysort.cu).
constexpr size_t RAY_SORT_MIN = 1 << 16;

template <bool COUNT>
cudaError_t launch_rays(const vox_cuda_tree *t, const float *o, const float *d, const uint32_t *roots,
                        size_t n, uint32_t *leaf, uint8_t *slot, float *pts,
                        unsigned long long *counts, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    void *scratch = nullptr;
    uint32_t *order = nullptr;
    if (!COUNT && n >= RAY_SORT_MIN && n <= 0xFFFFFFFFull) {
        cudaError_t e = cudaMallocAsync(&scratch, ray_order_bytes(n), s);
        if (e != cudaSuccess) return e;
        e = ray_order(t, o, d, n, scratch, &order, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(scratch, s);
            return e;
        }
    }
    dim3 block(256), grid((unsigned)((n + 255) / 256));
    switch (t->cap_class) {
    case 0: ray_kernel<CAP0, COUNT><<<grid, block, 0, s>>>(t->dev, o, d, roots, n, leaf, slot, pts, counts, t->d_status, order); break;
    case 1: ray_kernel<CAP1, COUNT><<<grid, block, 0, s>>>(t->dev, o, d, roots, n, leaf, slot, pts, counts, t->d_status, order); break;
    default: ray_kernel<CAP2, COUNT><<<grid, block, 0, s>>>(t->dev, o, d, roots, n, leaf, slot, pts, counts, t->d_status, order); break;
    }
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (scratch) cudaFreeAsync(scratch, s);
    return e;
}

// Batches of at least this many balls are searched grouped by centre cell.
constexpr size_t BALL_SORT_MIN = 1 << 18;

template <bool COUNT>
cudaError_t launch_balls(const vox_cuda_tree *t, const float *c, const float *r, size_t n, uint8_t *hit,
                         unsigned long long *counts, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    void *scratch = nullptr;
    uint32_t *order = nullptr;
    if (!COUNT && n >= BALL_SORT_MIN && n <= 0xFFFFFFFFull) {
        cudaError_t e = cudaMallocAsync(&scratch, ray_order_bytes(n), s);
        if (e != cudaSuccess) return e;
        e = ball_order(t, c, n, scratch, &order, s);
        if (e != cudaSuccess) {
            cudaFreeAsync(scratch, s);
            return e;
        }
    }
    dim3 block(256), grid((unsigned)((n + 255) / 256));
    switch (t->cap_class) {
    case 0: ball_kernel<CAP0, COUNT><<<grid, block, 0, s>>>(t->dev, c, r, n, hit, counts, t->d_status, order); break;
    case 1: ball_kernel<CAP1, COUNT><<<grid, block, 0, s>>>(t->dev, c, r, n, hit, counts, t->d_status, order); break;
    default: ball_kernel<CAP2, COUNT><<<grid, block, 0, s>>>(t->dev, c, r, n, hit, counts, t->d_status, order); break;
    }
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (scratch) cudaFreeAsync(scratch, s);
    return e;
}

// Process-wide settings of the BEST frame kernel (vox_cuda_render_set_config).
std::atomic<uint32_t> g_render_cull{1}, g_render_overlap{1};

// Two builds of the frame kernel draw the same frame.  A frame that is
// waited for on its own (the host-buffer calls) is bound by its slowest
// warps, which run fastest with the registers they want (8 blocks per SM).
// Frames enqueued back to back (the device calls) overlap one another, and
// there more warps per SM hide more latency: 12 blocks per SM, at the cost of
// a few spilled registers.
constexpr int MINB_ALONE = 8, MINB_PIPELINED = 12;

template <bool COUNT>
cudaError_t launch_render(const vox_cuda_tree *t, const vox_cuda_camera &cam, uint32_t w, uint32_t h,
                          const uint8_t *tex, uint32_t *argb, unsigned long long *counts, cudaStream_t s,
                          bool pipelined = false, const vox::DevLights *lights = nullptr,
                          vox::FrameMemo *memo = nullptr)
{
    // the counting kernel counts the reference's work: every pixel traced
    FramePlan p;
    plan_frame(t, cam, w, h, !COUNT && g_render_cull.load(), p);
    if (memo) plan_clearing(p, memo);
    void (*kern)(DevTree, vox_cuda_camera, uint32_t, uint32_t, FramePlan, const uint8_t *, uint32_t *,
                 unsigned long long *, uint32_t *, vox::DevLights);
    vox::DevLights L{};
    if (lights) L = *lights;
    const bool lit = !COUNT && L.on;
    const int cap = t->cap_class;
    if (lit) {
        if (pipelined) kern = cap == 0 ? render_kernel<CAP0, COUNT, MINB_PIPELINED, true>
                            : cap == 1 ? render_kernel<CAP1, COUNT, MINB_PIPELINED, true>
                                       : render_kernel<CAP2, COUNT, MINB_PIPELINED, true>;
        else kern = cap == 0 ? render_kernel<CAP0, COUNT, MINB_ALONE, true>
                  : cap == 1 ? render_kernel<CAP1, COUNT, MINB_ALONE, true>
                             : render_kernel<CAP2, COUNT, MINB_ALONE, true>;
    } else if (pipelined && !COUNT) {
        kern = cap == 0 ? render_kernel<CAP0, COUNT, MINB_PIPELINED, false>
             : cap == 1 ? render_kernel<CAP1, COUNT, MINB_PIPELINED, false>
                        : render_kernel<CAP2, COUNT, MINB_PIPELINED, false>;
    } else {
        kern = cap == 0 ? render_kernel<CAP0, COUNT, MINB_ALONE, false>
             : cap == 1 ? render_kernel<CAP1, COUNT, MINB_ALONE, false>
                        : render_kernel<CAP2, COUNT, MINB_ALONE, false>;
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.ntiles + p.nclear);
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = g_render_overlap.load() ? 1 : 0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, kern, t->dev, cam, w, h, p, tex, argb, counts, t->d_status, L);
    count_launch();
    if (e == cudaSuccess) e = cudaGetLastError();
    if (memo) *memo = FrameMemo{e == cudaSuccess, p.x0, p.y0, p.x1, p.y1};
    return e;
}

// FAST / ADAPTIVE frames, and with a ray buffer frames of every quality: one
// launch over the squares of the rectangle where rays can meet the tree,
// with blocks that clear the rest of the frame.
cudaError_t launch_render_squares(const vox_cuda_tree *t, const vox_cuda_camera &cam, uint32_t w, uint32_t h,
                                  unsigned int quality, const uint8_t *tex, uint32_t *argb, cudaStream_t s,
                                  const vox::DevLights *lights = nullptr, const float *rays = nullptr,
                                  vox::FrameMemo *memo = nullptr)
{
    vox::DevLights L{};
    if (lights) L = *lights;
    // the rectangle where rays can meet the tree's box, whole 4x4 squares,
    // and clearing blocks for the rest of the frame (a camera class the
    // device does not know, whose rays come in a buffer: the whole frame)
    FramePlan p;
    if (!rays) {
        plan_frame(t, cam, w, h, g_render_cull.load() != 0, p);
    } else {
        p.x0 = p.y0 = 0;
        p.x1 = w;
        p.y1 = h;
        p.ntx = (w + TILE_W - 1) / TILE_W;
        p.nty = (h + TILE_H - 1) / TILE_H;
        p.ctx = p.ntx / 2;
        p.cty = p.nty / 2;
        p.ntiles = p.ntx * p.nty;
        p.nclear = 0;
        p.cx0 = p.cy0 = 0;
        p.cx1 = w;
        p.cy1 = h;
    }
    if (memo) plan_clearing(p, memo);
    const int cap = t->cap_class;
    void (*squares)(DevTree, vox_cuda_camera, uint32_t, uint32_t, FramePlan, unsigned int, const uint8_t *,
                    uint32_t *, uint32_t *, vox::DevLights, const float *);
    if (rays)
        squares = cap == 0 ? render_squares_kernel<CAP0, true>
                : cap == 1 ? render_squares_kernel<CAP1, true> : render_squares_kernel<CAP2, true>;
    else
        squares = cap == 0 ? render_squares_kernel<CAP0, false>
                : cap == 1 ? render_squares_kernel<CAP1, false> : render_squares_kernel<CAP2, false>;
    // overlapping the previous kernel of the stream, as the BEST frames do
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(p.ntiles + p.nclear);
    cfg.blockDim = dim3(128);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = g_render_overlap.load() ? 1 : 0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, squares, t->dev, cam, w, h, p, quality, tex, argb, t->d_status, L, rays);
    count_launch();
    if (e == cudaSuccess) e = cudaGetLastError();
    if (memo) *memo = FrameMemo{e == cudaSuccess, p.x0, p.y0, p.x1, p.y1};
    return e;
}


// The error a nonzero status word reports.
int status_error(uint32_t st)
{
    return (st & vox::VOX_STATUS_RANGE) ? VOX_CUDA_ERANGE : VOX_CUDA_ESTACK;
}

// Reads and clears the tree's overflow flag after a synchronous call.
int check_tree_status(const vox_cuda_tree *t, cudaStream_t s)
{
    uint32_t st = 0;
    if (cudaMemcpyAsync(&st, t->d_status, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess) return VOX_CUDA_ECUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return VOX_CUDA_ECUDA;
    if (st) {
        cudaMemsetAsync(t->d_status, 0, 4, s);
        cudaStreamSynchronize(s);
        return status_error(st);
    }
    return VOX_CUDA_OK;
}

// Stream-ordered scratch for the host-buffer entry points.
struct Scratch {
    cudaStream_t s;
    void *p = nullptr;
    explicit Scratch(cudaStream_t st) : s(st) {}
    cudaError_t get(size_t bytes) { return cudaMallocAsync(&p, bytes ? bytes : 16, s); }
    ~Scratch() { if (p) cudaFreeAsync(p, s); }
};

inline size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

void count_launch() { g_launches++; }



// Linear map of screen2world: direction = M * (mul*sx - xsub, 1, ysub' - mul*sy)
// with ysub' = ysub for the simple camera (quaternion rotation, every term of
// which is linear in the vector) and ysub + k for the doom camera (rotation
// by phi about z).  Returns false for a camera whose state is not finite.
static bool camera_map(const vox_cuda_camera &cam, double M[3][3], double &ysub)
{
    const float f[] = {cam.position[0], cam.position[1], cam.position[2], cam.rotation[0], cam.rotation[1],
                       cam.rotation[2], cam.rotation[3], cam.mul, cam.xsub, cam.ysub, cam.sinphi,
                       cam.cosphi, cam.k};
    for (float x : f)
        if (!std::isfinite(x)) return false;
    ysub = cam.ysub;
    if (cam.kind == VOX_CUDA_CAMERA_DOOM) {
        double c = cam.cosphi, sn = cam.sinphi;
        double D[3][3] = {{c, -sn, 0}, {sn, c, 0}, {0, 0, 1}};
        std::memcpy(M, D, sizeof D);
        ysub += cam.k;
        return true;
    }
    double qw = cam.rotation[0], qi = cam.rotation[1], qj = cam.rotation[2], qk = cam.rotation[3];
    for (int j = 0; j < 3; j++) {
        double v[3] = {0, 0, 0};
        v[j] = 1;
        double t0 = 2 * (qj * v[2] - qk * v[1]), t1 = 2 * (qk * v[0] - qi * v[2]), t2 = 2 * (qi * v[1] - qj * v[0]);
        M[0][j] = v[0] + qw * t0 + (qj * t2 - qk * t1);
        M[1][j] = v[1] + qw * t1 + (qk * t0 - qi * t2);
        M[2][j] = v[2] + qw * t2 + (qi * t1 - qj * t0);
    }
    return true;
}

// The rectangle of a frame that can see the box bbox (min xyz, max xyz).
// The eight corners of the box, widened by a margin far above the rounding
// of the float search, are projected through the inverse of the camera map;
// the pixels whose rays can enter the box lie in the convex hull of the
// projections (the rays of a frame are an affine family of directions from
// one point), so the rectangle around them, widened by two pixels plus the
// rounding of the float ray directions, holds every pixel that can hit.  A
// box wholly behind the camera plane gives no pixel (every ray points
// forward); one with a corner at or behind the plane (the camera in or next
// to the box), a degenerate or non-finite camera give the whole frame.  The rectangle is
// rounded out to multiples of 8 x 4 pixels; [0,0)x[0,0) when no pixel can
// see the box.  centre_px receives where the box's centre projects (the
// frame centre when it lies behind the camera).
static void frame_rect(const float bbox[6], const vox_cuda_camera &cam, uint32_t w, uint32_t h,
                       uint32_t rect[4], double centre_px[2])
{
    uint32_t x0 = 0, y0 = 0, x1 = w, y1 = h;
    centre_px[0] = 0.5 * w;
    centre_px[1] = 0.5 * h;
    bool empty = false;
    double M[3][3], ysub = 0;
    if (camera_map(cam, M, ysub) && cam.mul != 0.0f && std::isfinite(bbox[0] + bbox[1] + bbox[2] +
                                                                    bbox[3] + bbox[4] + bbox[5])) {
        double det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) -
                     M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                     M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
        double nm = 0;
        for (auto &r : M)
            for (double x : r) nm += x * x;
        if (std::fabs(det) > 1e-9 * nm * std::sqrt(nm)) {
            double Mi[3][3];
            Mi[0][0] = (M[1][1] * M[2][2] - M[1][2] * M[2][1]) / det;
            Mi[0][1] = (M[0][2] * M[2][1] - M[0][1] * M[2][2]) / det;
            Mi[0][2] = (M[0][1] * M[1][2] - M[0][2] * M[1][1]) / det;
            Mi[1][0] = (M[1][2] * M[2][0] - M[1][0] * M[2][2]) / det;
            Mi[1][1] = (M[0][0] * M[2][2] - M[0][2] * M[2][0]) / det;
            Mi[1][2] = (M[0][2] * M[1][0] - M[0][0] * M[1][2]) / det;
            Mi[2][0] = (M[1][0] * M[2][1] - M[1][1] * M[2][0]) / det;
            Mi[2][1] = (M[0][1] * M[2][0] - M[0][0] * M[2][1]) / det;
            Mi[2][2] = (M[0][0] * M[1][1] - M[0][1] * M[1][0]) / det;
            double nmi = 0;
            for (auto &r : Mi)
                for (double x : r) nmi += x * x;
            const double o[3] = {cam.position[0], cam.position[1], cam.position[2]};
            double big = 1.0;
            for (int i = 0; i < 3; i++)
                big = std::max({big, std::fabs(o[i]), std::fabs((double)bbox[i]), std::fabs((double)bbox[3 + i])});
            const double mw = 1e-4 * big;                        // world margin
            const double mul = cam.mul, xsub = cam.xsub;
            const double vmax = 1 + std::fabs(xsub) + std::fabs(ysub) + std::fabs(mul) * ((double)w + h);
            const double mpx = 2 + 1e-5 * vmax * std::sqrt(nm * nmi) / std::fabs(mul);   // pixel margin
            double sxmin = INFINITY, sxmax = -INFINITY, symin = INFINITY, symax = -INFINITY;
            bool bounded = true;
            int behind = 0;
            for (int c = 0; c < 8; c++) {
                double P[3], a[3];
                for (int i = 0; i < 3; i++)
                    P[i] = ((c >> i) & 1) ? (double)bbox[3 + i] + mw : (double)bbox[i] - mw;
                for (int i = 0; i < 3; i++)
                    a[i] = Mi[i][0] * (P[0] - o[0]) + Mi[i][1] * (P[1] - o[1]) + Mi[i][2] * (P[2] - o[2]);
                double na = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
                if (a[1] < -1e-6 * na) behind++;
                if (!(a[1] > 1e-6 * na)) { bounded = false; continue; }
                double sx = (a[0] / a[1] + xsub) / mul, sy = (ysub - a[2] / a[1]) / mul;
                sxmin = std::min(sxmin, sx); sxmax = std::max(sxmax, sx);
                symin = std::min(symin, sy); symax = std::max(symax, sy);
            }
            if (behind == 8) {
                empty = true;          // the whole box lies behind the camera plane
            } else if (bounded && std::isfinite(sxmin + sxmax + symin + symax)) {
                double xa = std::floor(sxmin - mpx), xb = std::ceil(sxmax + mpx);
                double ya = std::floor(symin - mpx), yb = std::ceil(symax + mpx);
                if (xb < 0 || yb < 0 || xa > w - 1.0 || ya > h - 1.0) {
                    empty = true;
                } else {
                    xa = std::max(xa, 0.0); ya = std::max(ya, 0.0);
                    xb = std::min(xb, w - 1.0); yb = std::min(yb, h - 1.0);
                    x0 = (uint32_t)xa & ~7u; y0 = (uint32_t)ya & ~3u;
                    x1 = std::min(w, ((uint32_t)xb & ~7u) + 8u);
                    y1 = std::min(h, ((uint32_t)yb & ~3u) + 4u);
                }
            }
            double C[3], a[3];
            for (int i = 0; i < 3; i++) C[i] = 0.5 * ((double)bbox[i] + bbox[3 + i]) - o[i];
            for (int i = 0; i < 3; i++) a[i] = Mi[i][0] * C[0] + Mi[i][1] * C[1] + Mi[i][2] * C[2];
            if (a[1] > 1e-9) {
                centre_px[0] = (a[0] / a[1] + xsub) / mul;
                centre_px[1] = (ysub - a[2] / a[1]) / mul;
            }
        }
    }
    if (empty) x0 = x1 = y0 = y1 = 0;
    rect[0] = x0; rect[1] = y0; rect[2] = x1; rect[3] = y1;
}

void plan_frame(const vox_cuda_tree *t, const vox_cuda_camera &cam, uint32_t w, uint32_t h, bool cull,
                FramePlan &p)
{
    uint32_t r[4] = {0, 0, w, h};
    double c[2] = {0.5 * w, 0.5 * h};
    if (t->dev.root == VOXP_EMPTY) {
        if (cull) r[2] = r[3] = 0;
    } else {
        frame_rect(t->bbox, cam, w, h, r, c);
        if (!cull) { r[0] = r[1] = 0; r[2] = w; r[3] = h; }
    }
    p.x0 = r[0]; p.y0 = r[1]; p.x1 = r[2]; p.y1 = r[3];
    p.ntx = (p.x1 - p.x0 + TILE_W - 1) / TILE_W;
    p.nty = (p.y1 - p.y0 + TILE_H - 1) / TILE_H;
    p.ntiles = p.ntx * p.nty;
    double tx = (c[0] - p.x0) / TILE_W, ty = (c[1] - p.y0) / TILE_H;
    p.ctx = (p.ntx && tx >= 0) ? (uint32_t)std::min(tx, p.ntx - 1.0) : 0;   // NaN -> 0
    p.cty = (p.nty && ty >= 0) ? (uint32_t)std::min(ty, p.nty - 1.0) : 0;
    p.cx0 = 0; p.cy0 = 0; p.cx1 = w; p.cy1 = h;
    plan_clearing(p, nullptr);
}

// The clearing blocks of a plan: the frame outside the traced rectangle, or
// with a valid memo only the part of the memo's rectangle outside it; one
// warp a row, up to 64 blocks, none when nothing is left (a launch with no
// tracing block still gets one block, which finds nothing to do).
void plan_clearing(FramePlan &p, const FrameMemo *memo)
{
    if (memo && memo->valid) {
        p.cx0 = memo->x0; p.cy0 = memo->y0; p.cx1 = memo->x1; p.cy1 = memo->y1;
    }
    const bool empty = p.cx1 <= p.cx0 || p.cy1 <= p.cy0;
    const bool covered = p.x1 > p.x0 && p.y1 > p.y0 && p.cx0 >= p.x0 && p.cx1 <= p.x1 && p.cy0 >= p.y0 &&
                         p.cy1 <= p.y1;
    p.nclear = (empty || covered) ? 0u : std::min<uint32_t>(64u, (p.cy1 - p.cy0 + 3) / 4);
    if (p.ntiles + p.nclear == 0) p.nclear = 1;
}

void frame_rect_of(const vox_cuda_tree *t, const vox_cuda_camera &cam, uint32_t w, uint32_t h, uint32_t rect[4],
                   double centre_px[2])
{
    if (t->dev.root == VOXP_EMPTY) {
        rect[0] = rect[1] = rect[2] = rect[3] = 0;
        centre_px[0] = 0.5 * w;
        centre_px[1] = 0.5 * h;
        return;
    }
    frame_rect(t->bbox, cam, w, h, rect, centre_px);
}

// ======================================================================== API

EXPORT const char *vox_cuda_strerror(int code)
try {
    switch (code) {
    case VOX_CUDA_OK: return "ok";
    case VOX_CUDA_EINVAL: return "invalid argument";
    case VOX_CUDA_ENOMEM: return "out of memory";
    case VOX_CUDA_ECUDA: return "CUDA runtime error";
    case VOX_CUDA_EDEPTH: return "tree deeper than the traversal stack supports";
    case VOX_CUDA_ESTACK: return "traversal stack overflow";
    case VOX_CUDA_ETOOBIG: return "flattened tree exceeds the pool limit";
    case VOX_CUDA_EGEOMETRY: return "frame width must be a multiple of 16 and height of 4";
    case VOX_CUDA_EBUDGET: return "admission budget exceeded";
    case VOX_CUDA_ETIMEOUT: return "bounded wait timed out";
    case VOX_CUDA_ENODEV: return "no CUDA device";
    case VOX_CUDA_ECAPACITY: return "request exceeds the entry point's fixed capacity";
    case VOX_CUDA_ERANGE: return "a search met an index outside the uploaded tree (checked build)";
    default: return "unknown error";
    }
} VOX_ABI_FAIL_NULL

EXPORT const char *vox_cuda_version(void) { return "voxtrees_cuda 0.1 (sm_103a)"; }

namespace {

// Reads `n16` 16-byte units `reps` times over, bypassing L1 (ld.global.cg),
// so that every load is served by L2 while the buffer fits it.  The xor of
// everything read is stored only if it takes one particular value, which
// keeps the loads without writing anything in practice.
__global__ void __launch_bounds__(256) l2_read_kernel(const uint4 *__restrict__ buf, size_t n16, uint32_t reps,
                                                      uint32_t *__restrict__ sink)
{
    uint32_t acc = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    const size_t first = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t r = 0; r < reps; r++) {
        for (size_t i = first; i < n16; i += stride) {
            uint4 v = __ldcg(buf + i);
            acc ^= v.x ^ v.y ^ v.z ^ v.w;
        }
    }
    if (acc == 0x9E3779B9u) sink[0] = acc;
}

}  // namespace

EXPORT int vox_cuda_measure_l2_read(size_t bytes, uint32_t reps, float *gbs)
try {
    if (!gbs || bytes < 4096 || reps == 0) return VOX_CUDA_EINVAL;
    *gbs = 0.0f;
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return VOX_CUDA_ENODEV;
    const size_t n16 = bytes / 16;
    uint4 *buf = nullptr;
    uint32_t *sink = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    int rc = VOX_CUDA_ECUDA;
    if (cudaMalloc(&buf, n16 * 16) != cudaSuccess || cudaMalloc(&sink, 4) != cudaSuccess) {
        rc = VOX_CUDA_ENOMEM;
    } else if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess &&
               cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess &&
               cudaMemsetAsync(buf, 0x5A, n16 * 16, s) == cudaSuccess) {
        const dim3 grid(nsm * 8), block(256);
        l2_read_kernel<<<grid, block, 0, s>>>(buf, n16, 2, sink);   // warm: the buffer into L2
        count_launch();
        cudaEventRecord(e0, s);
        l2_read_kernel<<<grid, block, 0, s>>>(buf, n16, reps, sink);
        count_launch();
        cudaEventRecord(e1, s);
        float ms = 0.0f;
        if (cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess && ms > 0) {
            *gbs = (float)((double)n16 * 16.0 * reps / (ms * 1e-3) / 1e9);
            rc = VOX_CUDA_OK;
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (s) cudaStreamDestroy(s);
    cudaFree(buf);
    cudaFree(sink);
    return rc;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_build_checked(void) { return vox::CHECKED ? 1 : 0; }

EXPORT uint64_t vox_cuda_launch_count(void) { return g_launches.load(); }

// Flattens `root` into t (host maps) and copies the image to the device,
// reusing t's device buffers when they are large enough.  On failure t keeps
// its previous contents when `keep` is set (a refresh), else is left empty.
// The image of `root` read in the given vox_dot layout, with `voxel` (NULL:
// the library's vox_voxel) as the voxel size.
static int flatten_as(const struct vox_node *root, int layout, const float *voxel, FlatTree *f)
{
    const float *v = voxel ? voxel : vox_voxel;
    if (layout == VOX_CUDA_LAYOUT_SSE) return vox_flatten16(reinterpret_cast<const vox_node16 *>(root), v, f);
    return vox_flatten(root, v, f);
}

static int load_tree(vox_cuda_tree *t, const struct vox_node *root, int layout = VOX_CUDA_LAYOUT_SCALAR,
                     const float *voxel = nullptr)
{
    FlatTree flat;
    int rc = flatten_as(root, layout, voxel, &flat);
    if (rc == -2 || rc == -1) return VOX_CUDA_ETOOBIG;
    if (vox_flatten_validate(flat) != 0) return VOX_CUDA_EINVAL;
    int cls = cap_class_for_depth(flat.depth);
    if (cls < 0) return VOX_CUDA_EDEPTH;
    size_t units = flat.units.size() ? flat.units.size() : VOXP_REC_UNITS;
    size_t nodes = flat.preorder.size();
    size_t pool_bytes = units * 16, map_bytes = (nodes ? nodes : 1) * 4;
    uint4 *pool = t->d_pool;
    uint32_t *map = t->d_rec_of_id;
    bool new_pool = !pool || t->pool_bytes < pool_bytes, new_map = !map || t->map_bytes < map_bytes;
    if (new_pool && cudaMalloc(&pool, pool_bytes) != cudaSuccess) return VOX_CUDA_ENOMEM;
    if (new_map && cudaMalloc(&map, map_bytes) != cudaSuccess) {
        if (new_pool) cudaFree(pool);
        return VOX_CUDA_ENOMEM;
    }
    if (!t->d_status && cudaMalloc(&t->d_status, 4) != cudaSuccess) {
        if (new_pool) cudaFree(pool);
        if (new_map) cudaFree(map);
        return VOX_CUDA_ENOMEM;
    }
    cudaError_t e = cudaMemset(t->d_status, 0, 4);
    if (e == cudaSuccess && flat.units.size())
        e = cudaMemcpy(pool, flat.units.data(), flat.units.size() * 16, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nodes) e = cudaMemcpy(map, flat.rec_of_id.data(), nodes * 4, cudaMemcpyHostToDevice);
    // A copy from pageable memory may still be in flight when cudaMemcpy
    // returns; the pool must be complete before any kernel on any stream
    // reads it (the frame kernel reads it ahead of its stream dependency).
    if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamLegacy);
    if (e != cudaSuccess) {
        if (new_pool) cudaFree(pool);
        if (new_map) cudaFree(map);
        return VOX_CUDA_ECUDA;
    }
    if (new_pool) {
        if (t->d_pool) cudaFree(t->d_pool);
        t->d_pool = pool;
        t->pool_bytes = pool_bytes;
    }
    if (new_map) {
        if (t->d_rec_of_id) cudaFree(t->d_rec_of_id);
        t->d_rec_of_id = map;
        t->map_bytes = map_bytes;
    }
    t->cap_class = cls;
    if (root) {   // the root record: {min.xyz, max.x}, {max.yz, ...}
        const uint4_host &a = flat.units[0], &b = flat.units[1];
        const uint32_t bits[6] = {a.x, a.y, a.z, a.w, b.x, b.y};
        for (int i = 0; i < 6; i++) std::memcpy(&t->bbox[i], &bits[i], 4);
    } else {
        for (int i = 0; i < 6; i++) t->bbox[i] = 0.0f;
    }
    t->dev.pool = t->d_pool;
    t->dev.rec_of_id = t->d_rec_of_id;
    t->dev.root = root ? 0u : VOXP_EMPTY;
    t->dev.n_nodes = (uint32_t)nodes;
    t->dev.vx = flat.voxel[0];
    t->dev.vy = flat.voxel[1];
    t->dev.vz = flat.voxel[2];
    uint64_t steps = (uint64_t)nodes + flat.n_dots + 2;
    t->dev.max_steps = steps > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)steps;
    t->dev.n_units = (uint32_t)units;
    t->dev.fault = t->d_status;
    t->n_nodes = nodes;
    t->n_units = flat.units.size();
    // The flattened image is on the device now; keep only the maps.
    std::vector<uint4_host>().swap(flat.units);
    t->flat = std::move(flat);
    std::lock_guard<std::mutex> lock(t->index_mu);
    t->index.clear();
    t->index_built = false;
    return VOX_CUDA_OK;
}

int adopt_image(vox_cuda_tree *t, uint4 *pool, size_t pool_bytes, uint32_t *map, size_t map_bytes,
                const ImageStats &st)
{
    int cls = cap_class_for_depth(st.depth);
    if (cls < 0) return VOX_CUDA_EDEPTH;
    bool empty = st.nodes == 0;
    uint4 *own_pool = nullptr;
    uint32_t *own_map = nullptr;
    if (empty) {   // as the upload of a NULL tree: one record's worth of pool, a one-entry map
        pool_bytes = VOXP_REC_UNITS * 16;
        map_bytes = 4;
        if (cudaMalloc(&own_pool, pool_bytes) != cudaSuccess) return VOX_CUDA_ENOMEM;
        if (cudaMalloc(&own_map, map_bytes) != cudaSuccess) {
            cudaFree(own_pool);
            return VOX_CUDA_ENOMEM;
        }
        pool = own_pool;
        map = own_map;
    }
    if ((!t->d_status && cudaMalloc(&t->d_status, 4) != cudaSuccess) || cudaMemset(t->d_status, 0, 4) != cudaSuccess) {
        cudaFree(own_pool);
        cudaFree(own_map);
        return VOX_CUDA_ENOMEM;
    }
    if (t->d_pool) cudaFree(t->d_pool);
    if (t->d_rec_of_id) cudaFree(t->d_rec_of_id);
    t->d_pool = pool;
    t->pool_bytes = pool_bytes;
    t->d_rec_of_id = map;
    t->map_bytes = map_bytes;
    t->cap_class = cls;
    for (int i = 0; i < 6; i++) t->bbox[i] = empty ? 0.0f : st.bbox[i];
    t->dev.pool = pool;
    t->dev.rec_of_id = map;
    t->dev.root = empty ? VOXP_EMPTY : 0u;
    t->dev.n_nodes = (uint32_t)st.nodes;
    t->dev.vx = st.voxel[0];
    t->dev.vy = st.voxel[1];
    t->dev.vz = st.voxel[2];
    uint64_t steps = st.nodes + st.dots + 2;
    t->dev.max_steps = steps > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)steps;
    t->dev.n_units = (uint32_t)(empty ? VOXP_REC_UNITS : st.units);
    t->dev.fault = t->d_status;
    t->n_nodes = st.nodes;
    t->n_units = empty ? 0 : st.units;
    FlatTree f;
    f.n_inner = st.inner;
    f.n_leaf = st.leaf;
    f.n_dense = st.dense;
    f.n_dots = st.dots;
    f.depth = st.depth;
    for (int i = 0; i < 3; i++) f.voxel[i] = st.voxel[i];
    t->flat = std::move(f);
    std::lock_guard<std::mutex> lock(t->index_mu);
    t->index.clear();
    t->index_built = false;
    return VOX_CUDA_OK;
}

// dropin_search.cpp: a device copy vox_make_tree kept for the tree at `root`.
vox_cuda_tree *dropin_take_prebuilt(const vox_node *root);

bool tree_fits_now(const vox_cuda_tree *t)
{
    int dev = -1;
    return cudaGetDevice(&dev) == cudaSuccess && dev == t->device && t->flat.voxel[0] == vox_voxel[0] &&
           t->flat.voxel[1] == vox_voxel[1] && t->flat.voxel[2] == vox_voxel[2];
}

EXPORT int vox_cuda_tree_upload(const struct vox_node *root, vox_cuda_tree **out)
try {
    if (!out) return VOX_CUDA_EINVAL;
    if (root) {
        if (vox_cuda_tree *t = dropin_take_prebuilt(root)) {   // built on the GPU by vox_make_tree
            *out = t;
            return VOX_CUDA_OK;
        }
    }
    return tree_upload_flat(root, out);
} VOX_ABI_FAIL_INT

static int upload_as(const struct vox_node *root, int layout, const float *voxel, vox_cuda_tree **out)
{
    if (!out) return VOX_CUDA_EINVAL;
    *out = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return VOX_CUDA_ENODEV;
    vox_cuda_tree *t = new (std::nothrow) vox_cuda_tree();
    if (!t) return VOX_CUDA_ENOMEM;
    t->device = dev;
    int rc = load_tree(t, root, layout, voxel);
    if (rc) {
        cudaFree(t->d_pool);
        cudaFree(t->d_rec_of_id);
        cudaFree(t->d_status);
        delete t;
        return rc;
    }
    *out = t;
    return VOX_CUDA_OK;
}

int tree_upload_flat(const struct vox_node *root, vox_cuda_tree **out)
{
    return upload_as(root, VOX_CUDA_LAYOUT_SCALAR, nullptr, out);
}

static bool known_layout(int layout) { return layout == VOX_CUDA_LAYOUT_SCALAR || layout == VOX_CUDA_LAYOUT_SSE; }

EXPORT int vox_cuda_tree_upload_layout(const struct vox_node *root, int layout, const float *voxel,
                                       vox_cuda_tree **out)
try {
    if (!out || !known_layout(layout)) return VOX_CUDA_EINVAL;
    return upload_as(root, layout, voxel, out);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_refresh(vox_cuda_tree *t, const struct vox_node *root)
try {
    if (!t) return VOX_CUDA_EINVAL;
    // kernels in flight on any stream may still read the old image
    if (cudaDeviceSynchronize() != cudaSuccess) return VOX_CUDA_ECUDA;
    return load_tree(t, root);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_refresh_layout(vox_cuda_tree *t, const struct vox_node *root, int layout,
                                        const float *voxel)
try {
    if (!t || !known_layout(layout)) return VOX_CUDA_EINVAL;
    if (cudaDeviceSynchronize() != cudaSuccess) return VOX_CUDA_ECUDA;
    return load_tree(t, root, layout, voxel);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_measure(const struct vox_node *root, vox_cuda_tree_info *info)
try {
    if (!info) return VOX_CUDA_EINVAL;
    FlatTree f;
    int rc = vox_flatten(root, vox_voxel, &f);
    if (rc) return VOX_CUDA_ETOOBIG;
    if (vox_flatten_validate(f) != 0) return VOX_CUDA_EINVAL;
    if (cap_class_for_depth(f.depth) < 0) return VOX_CUDA_EDEPTH;
    info->nodes = f.preorder.size();
    info->inner = f.n_inner;
    info->leaves = f.n_leaf;
    info->dense_leaves = f.n_dense;
    info->dots = f.n_dots;
    info->depth = f.depth;
    info->device_bytes = (f.units.size() ? f.units.size() : VOXP_REC_UNITS) * 16 + 4 * f.preorder.size() + 4;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_free(vox_cuda_tree *t)
try {
    if (!t) return VOX_CUDA_EINVAL;
    int cur = 0;
    cudaGetDevice(&cur);
    if (cur != t->device) cudaSetDevice(t->device);
    cudaFree(t->d_pool);
    cudaFree(t->d_rec_of_id);
    cudaFree(t->d_status);
    if (cur != t->device) cudaSetDevice(cur);
    delete t;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_get_info(const vox_cuda_tree *t, vox_cuda_tree_info *info)
try {
    if (!t || !info) return VOX_CUDA_EINVAL;
    info->nodes = t->n_nodes;
    info->inner = t->flat.n_inner;
    info->leaves = t->flat.n_leaf;
    info->dense_leaves = t->flat.n_dense;
    info->dots = t->flat.n_dots;
    info->depth = t->flat.depth;
    info->device_bytes = t->pool_bytes + 4 * t->n_nodes + 4;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_image(const vox_cuda_tree *t, void *units, size_t units_cap, uint32_t *rec_of_id,
                               size_t ids_cap, size_t *n_units, size_t *n_ids)
try {
    if (!t) return VOX_CUDA_EINVAL;
    if (n_units) *n_units = t->n_units;
    if (n_ids) *n_ids = t->n_nodes;
    if ((units && units_cap < t->n_units) || (rec_of_id && ids_cap < t->n_nodes)) return VOX_CUDA_EINVAL;
    // kernels in flight on other streams may still write the status word only
    if (units && t->n_units &&
        cudaMemcpy(units, t->d_pool, t->n_units * 16, cudaMemcpyDeviceToHost) != cudaSuccess)
        return VOX_CUDA_ECUDA;
    if (rec_of_id && t->n_nodes &&
        cudaMemcpy(rec_of_id, t->d_rec_of_id, t->n_nodes * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
        return VOX_CUDA_ECUDA;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_flatten_host(const struct vox_node *root, void *units, size_t units_cap,
                                      uint32_t *rec_of_id, size_t ids_cap, size_t *n_units, size_t *n_ids)
try {
    return vox_cuda_tree_flatten_host_layout(root, VOX_CUDA_LAYOUT_SCALAR, nullptr, units, units_cap, rec_of_id,
                                             ids_cap, n_units, n_ids);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_flatten_host_layout(const struct vox_node *root, int layout, const float *voxel,
                                             void *units, size_t units_cap, uint32_t *rec_of_id, size_t ids_cap,
                                             size_t *n_units, size_t *n_ids)
try {
    if (!known_layout(layout)) return VOX_CUDA_EINVAL;
    FlatTree flat;
    int rc = flatten_as(root, layout, voxel, &flat);
    if (rc) return VOX_CUDA_ETOOBIG;
    const size_t nu = flat.units.size(), ni = flat.preorder.size();
    if (n_units) *n_units = nu;
    if (n_ids) *n_ids = ni;
    if ((units && units_cap < nu) || (rec_of_id && ids_cap < ni)) return VOX_CUDA_EINVAL;
    if (units && nu) std::memcpy(units, flat.units.data(), nu * 16);
    if (rec_of_id && ni) std::memcpy(rec_of_id, flat.rec_of_id.data(), ni * 4);
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_image_check(const void *units, size_t n_units, size_t n_nodes)
try {
    if (!units && n_units) return VOX_CUDA_EINVAL;
    FlatTree f;
    const uint4_host *u = static_cast<const uint4_host *>(units);
    if (n_units) f.units.assign(u, u + n_units);
    f.preorder.assign(n_nodes, nullptr);
    return vox_flatten_validate(f) == 0 ? VOX_CUDA_OK : VOX_CUDA_EINVAL;
} VOX_ABI_FAIL_INT

EXPORT const struct vox_node *vox_cuda_tree_node(const vox_cuda_tree *t, uint32_t id)
try {
    if (!t || id >= t->flat.preorder.size()) return nullptr;
    return t->flat.preorder[id];
} VOX_ABI_FAIL_NULL

EXPORT int vox_cuda_tree_node_id(const vox_cuda_tree *t, const struct vox_node *node, uint32_t *id)
try {
    if (!t || !id) return VOX_CUDA_EINVAL;
    vox_cuda_tree *m = const_cast<vox_cuda_tree *>(t);
    std::lock_guard<std::mutex> lock(m->index_mu);
    if (!m->index_built) {
        m->index.resize(t->flat.preorder.size());
        for (size_t i = 0; i < m->index.size(); i++) m->index[i] = {t->flat.preorder[i], (uint32_t)i};
        std::sort(m->index.begin(), m->index.end());
        m->index_built = true;
    }
    auto it = std::lower_bound(m->index.begin(), m->index.end(), std::make_pair(node, (uint32_t)0));
    if (it == m->index.end() || it->first != node) return VOX_CUDA_EINVAL;
    *id = it->second;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_ray_batch_device(const vox_cuda_tree *t, const float *o, const float *d,
                                     const uint32_t *roots, size_t n, uint32_t *leaf, uint8_t *slot,
                                     float *pts, void *stream)
try {
    if (!t || (n && (!o || !d || !leaf))) return VOX_CUDA_EINVAL;
    return status_of(launch_rays<false>(t, o, d, roots, n, leaf, slot, pts, nullptr, as_stream(stream)));
} VOX_ABI_FAIL_INT

// Host batches of up to SMALL_BATCH queries (the drop-in single queries
// among them) pass through a page-locked buffer of the calling thread that
// the kernel reads and writes in place: one launch and one synchronisation a
// call, with no device scratch and no copies (small_rays, small_balls).  A
// single vox_ray_tree_intersection on the 256^3 tree: 31 us against 54 us
// through device scratch and pageable copies; vox_tree_ball_collidep 30
// against 44 us; 256 rays 87 against 121 us.
static constexpr size_t SMALL_BATCH = 256;
static int small_rays(const vox_cuda_tree *t, const float *o, const float *d, const uint32_t *roots, size_t n,
                      uint32_t *leaf, uint8_t *slot, float *pts, cudaStream_t s);
static int small_balls(const vox_cuda_tree *t, const float *c, const float *r, size_t n, uint8_t *hit,
                       cudaStream_t s);

EXPORT int vox_cuda_ray_batch(const vox_cuda_tree *t, const float *o, const float *d,
                              const uint32_t *roots, size_t n, uint32_t *leaf, uint8_t *slot,
                              float *pts, void *stream)
try {
    if (!t || (n && (!o || !d || !leaf))) return VOX_CUDA_EINVAL;
    if (n == 0) return VOX_CUDA_OK;
    cudaStream_t s = as_stream(stream);
    if (n <= SMALL_BATCH) return small_rays(t, o, d, roots, n, leaf, slot, pts, s);
    size_t b_in = align256(n * 12), b_root = roots ? align256(n * 4) : 0;
    size_t b_leaf = align256(n * 4), b_slot = align256(n), b_pts = align256(n * 12);
    Scratch sc(s);
    if (sc.get(2 * b_in + b_root + b_leaf + b_slot + b_pts) != cudaSuccess) return VOX_CUDA_ENOMEM;
    char *base = static_cast<char *>(sc.p);
    float *d_o = reinterpret_cast<float *>(base);
    float *d_d = reinterpret_cast<float *>(base + b_in);
    uint32_t *d_roots = roots ? reinterpret_cast<uint32_t *>(base + 2 * b_in) : nullptr;
    uint32_t *d_leaf = reinterpret_cast<uint32_t *>(base + 2 * b_in + b_root);
    uint8_t *d_slot = reinterpret_cast<uint8_t *>(base + 2 * b_in + b_root + b_leaf);
    float *d_pts = reinterpret_cast<float *>(base + 2 * b_in + b_root + b_leaf + b_slot);
    cudaError_t e = cudaMemcpyAsync(d_o, o, n * 12, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_d, d, n * 12, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess && roots) e = cudaMemcpyAsync(d_roots, roots, n * 4, cudaMemcpyHostToDevice, s);
    // points are written on hits only: start from the caller's values
    if (e == cudaSuccess && pts) e = cudaMemcpyAsync(d_pts, pts, n * 12, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
        e = launch_rays<false>(t, d_o, d_d, d_roots, n, d_leaf, d_slot, pts ? d_pts : nullptr, nullptr, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(leaf, d_leaf, n * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && slot) e = cudaMemcpyAsync(slot, d_slot, n, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && pts) e = cudaMemcpyAsync(pts, d_pts, n * 12, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return VOX_CUDA_ECUDA;
    return check_tree_status(t, s);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_ball_batch_device(const vox_cuda_tree *t, const float *c, const float *r, size_t n,
                                      uint8_t *hit, void *stream)
try {
    if (!t || (n && (!c || !r || !hit))) return VOX_CUDA_EINVAL;
    return status_of(launch_balls<false>(t, c, r, n, hit, nullptr, as_stream(stream)));
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_ball_batch(const vox_cuda_tree *t, const float *c, const float *r, size_t n,
                               uint8_t *hit, void *stream)
try {
    if (!t || (n && (!c || !r || !hit))) return VOX_CUDA_EINVAL;
    if (n == 0) return VOX_CUDA_OK;
    cudaStream_t s = as_stream(stream);
    if (n <= SMALL_BATCH) return small_balls(t, c, r, n, hit, s);
    size_t b_c = align256(n * 12), b_r = align256(n * 4), b_h = align256(n);
    Scratch sc(s);
    if (sc.get(b_c + b_r + b_h) != cudaSuccess) return VOX_CUDA_ENOMEM;
    char *base = static_cast<char *>(sc.p);
    float *d_c = reinterpret_cast<float *>(base);
    float *d_r = reinterpret_cast<float *>(base + b_c);
    uint8_t *d_h = reinterpret_cast<uint8_t *>(base + b_c + b_r);
    cudaError_t e = cudaMemcpyAsync(d_c, c, n * 12, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_r, r, n * 4, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = launch_balls<false>(t, d_c, d_r, n, d_h, nullptr, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hit, d_h, n, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return VOX_CUDA_ECUDA;
    return check_tree_status(t, s);
} VOX_ABI_FAIL_INT

static int check_render_args(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                             const uint8_t *tex, const uint32_t *argb)
{
    if (!t || !cam || !tex || !argb) return VOX_CUDA_EINVAL;
    if (cam->kind != VOX_CUDA_CAMERA_SIMPLE && cam->kind != VOX_CUDA_CAMERA_DOOM) return VOX_CUDA_EINVAL;
    if (w == 0 || h == 0 || (w & 0xF) || (h & 0x3)) return VOX_CUDA_EGEOMETRY;
    return VOX_CUDA_OK;
}

EXPORT int vox_cuda_render_device(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                                  const uint8_t *tex, uint32_t *argb, void *stream)
try {
    int rc = check_render_args(t, cam, w, h, tex, argb);
    if (rc) return rc;
    return status_of(launch_render<false>(t, *cam, w, h, tex, argb, nullptr, as_stream(stream), true));
} VOX_ABI_FAIL_INT

// Per host thread and device: what the synchronous host-buffer frame calls
// reuse from one call to the next.  A call returns only after its stream has
// finished with these, so the next call of the same thread may use them
// whatever stream it names.
struct HostCallState {
    uint8_t *d_tex = nullptr;      // device copy of the texture last used
    uint8_t *h_tex = nullptr;      // pinned: the bytes d_tex holds (valid if tex_ok)
    uint32_t *h_status = nullptr;  // pinned: the tree's status word read back
    bool tex_ok = false;
    unsigned char *h_small = nullptr;    // pinned, mapped: small batches' inputs and results (small_rays)
    unsigned char *d_small = nullptr;    // the device's address of h_small
    // vox_cuda_render_frames: device frames the kernels draw into, a stream
    // copying each finished frame out, and per slot "drawn" / "copied" events
    uint32_t *d_stage = nullptr;
    size_t stage_bytes = 0;
    uint32_t *d_zero = nullptr;          // device zeros, the source of copy_outside
    size_t zero_bytes = 0;
    uint32_t *d_frame = nullptr;         // the single-frame calls' device frame (host_call_frame)
    size_t frame_bytes = 0;
    unsigned char *h_tables = nullptr;   // pinned: one job table per chunk of frames
    size_t tables_bytes = 0;
    void *d_table = nullptr;             // device: the job table of the chunk being drawn, its queue head
    size_t d_table_bytes = 0;
    uint32_t *d_done = nullptr;          // device: finished items per frame of a launch
    uint32_t *h_flags = nullptr;         // pinned: per frame of a launch, the epoch once complete
    uint32_t *d_flags = nullptr;         // the device's address of h_flags
    size_t flags_n = 0;
    uint32_t epoch = 0;
    cudaStream_t copy = nullptr;
    std::vector<cudaEvent_t> drawn, copied;
    cudaEvent_t fin = nullptr;
    ~HostCallState()               // at thread exit; errors after the CUDA context is gone are moot
    {
        if (d_tex) cudaFree(d_tex);
        if (h_tex) cudaFreeHost(h_tex);
        if (d_stage) cudaFree(d_stage);
        if (d_zero) cudaFree(d_zero);
        if (d_frame) cudaFree(d_frame);
        if (h_tables) cudaFreeHost(h_tables);
        if (h_small) cudaFreeHost(h_small);
        if (d_table) cudaFree(d_table);
        if (d_done) cudaFree(d_done);
        if (h_flags) cudaFreeHost(h_flags);
        for (cudaEvent_t e : drawn) cudaEventDestroy(e);
        for (cudaEvent_t e : copied) cudaEventDestroy(e);
        if (fin) cudaEventDestroy(fin);
        if (copy) cudaStreamDestroy(copy);
    }
};

// Staging frames (`bytes` for `slots` frames), `tables` bytes of pinned job
// tables, a device job table of `table` bytes, completion counters and flags
// for `group` frames, and the copy stream with `zeros` bytes of device zeros
// (host_call_copies; all grow only).
static cudaError_t host_call_copies(HostCallState *hc, size_t zeros, cudaStream_t s);

static cudaError_t stage_reserve(HostCallState *hc, size_t bytes, uint32_t slots, size_t tables, size_t table,
                                 uint32_t group, size_t zeros, cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
    if (hc->flags_n < group) {
        if (hc->d_done || hc->h_flags) cudaDeviceSynchronize();
        if (hc->d_done) cudaFree(hc->d_done);
        if (hc->h_flags) cudaFreeHost(hc->h_flags);
        hc->d_done = nullptr;
        hc->h_flags = hc->d_flags = nullptr;
        hc->flags_n = 0;
        void *hp = nullptr, *dp = nullptr;
        e = cudaMalloc(&hc->d_done, group * sizeof(uint32_t));
        if (e == cudaSuccess) e = cudaMallocHost(&hp, group * sizeof(uint32_t));
        if (e == cudaSuccess) {
            std::memset(hp, 0, group * sizeof(uint32_t));
            e = cudaHostGetDevicePointer(&dp, hp, 0);
        }
        if (e == cudaSuccess) {
            hc->h_flags = static_cast<uint32_t *>(hp);
            hc->d_flags = static_cast<uint32_t *>(dp);
            hc->flags_n = group;
        } else {
            if (hc->d_done) cudaFree(hc->d_done);
            if (hp) cudaFreeHost(hp);
            hc->d_done = nullptr;
            return e;
        }
    }
    if (e == cudaSuccess) e = host_call_copies(hc, zeros, s);
    while (e == cudaSuccess && hc->drawn.size() < slots) {
        cudaEvent_t a = nullptr, b = nullptr;
        e = cudaEventCreateWithFlags(&a, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b, cudaEventDisableTiming);
        if (e != cudaSuccess) {
            if (a) cudaEventDestroy(a);
            break;
        }
        hc->drawn.push_back(a);
        hc->copied.push_back(b);
    }
    if (e == cudaSuccess && hc->tables_bytes < tables) {
        if (hc->h_tables) {
            cudaDeviceSynchronize();
            cudaFreeHost(hc->h_tables);
            hc->h_tables = nullptr;
            hc->tables_bytes = 0;
        }
        e = cudaMallocHost(&hc->h_tables, tables);
        if (e == cudaSuccess) hc->tables_bytes = tables;
        else hc->h_tables = nullptr;
    }
    if (e == cudaSuccess && hc->d_table_bytes < table + 256) {
        if (hc->d_table) {
            cudaDeviceSynchronize();
            cudaFree(hc->d_table);
            hc->d_table = nullptr;
            hc->d_table_bytes = 0;
        }
        e = cudaMalloc(&hc->d_table, table + 256);
        if (e == cudaSuccess) hc->d_table_bytes = table + 256;
        else hc->d_table = nullptr;
    }
    if (e == cudaSuccess && hc->stage_bytes < bytes) {
        if (hc->d_stage) {
            cudaDeviceSynchronize();   // an earlier call's copies may still read the old frames
            cudaFree(hc->d_stage);
            hc->d_stage = nullptr;
            hc->stage_bytes = 0;
        }
        e = cudaMalloc(&hc->d_stage, bytes);
        if (e == cudaSuccess) hc->stage_bytes = bytes;
        else hc->d_stage = nullptr;
    }
    return e;
}

static HostCallState *host_call_state()
{
    constexpr int MAXDEV = 64;
    thread_local HostCallState st[MAXDEV];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAXDEV) return nullptr;
    HostCallState &h = st[dev];
    if (!h.d_tex) {
        void *p = nullptr;
        if (cudaMallocHost(&p, 32768 + 256) != cudaSuccess) return nullptr;
        if (cudaMalloc(&h.d_tex, 32768) != cudaSuccess) {
            cudaFreeHost(p);
            h.d_tex = nullptr;
            return nullptr;
        }
        h.h_tex = static_cast<uint8_t *>(p);
        h.h_status = reinterpret_cast<uint32_t *>(static_cast<uint8_t *>(p) + 32768);
    }
    return &h;
}

// The calling thread's small-batch buffer: SMALL_BYTES of page-locked memory,
// mapped into the device's address space, in regions of 4 KiB (SMALL_BATCH
// rays' origins, directions, roots, points, leaf ids, slots; or balls'
// centres, radii, answers) and a status word.
static constexpr size_t SMALL_REGION = 4096, SMALL_BYTES = 8 * SMALL_REGION;
static_assert(SMALL_BATCH * 12 <= SMALL_REGION, "a region holds SMALL_BATCH points");

static bool small_buffer(HostCallState *hc)
{
    if (hc->h_small) return true;
    void *p = nullptr, *dp = nullptr;
    if (cudaHostAlloc(&p, SMALL_BYTES, cudaHostAllocMapped) != cudaSuccess) return false;
    if (cudaHostGetDevicePointer(&dp, p, 0) != cudaSuccess) {
        cudaFreeHost(p);
        return false;
    }
    hc->h_small = static_cast<unsigned char *>(p);
    hc->d_small = static_cast<unsigned char *>(dp);
    return true;
}

// The tree's status word into the small buffer's last region, the one
// synchronisation, then the status as vox_cuda_ray_batch reports it.
static int small_finish(HostCallState *hc, const vox_cuda_tree *t, cudaStream_t s, cudaError_t e)
{
    uint32_t *st = reinterpret_cast<uint32_t *>(hc->h_small + 7 * SMALL_REGION);
    if (e == cudaSuccess) e = cudaMemcpyAsync(st, t->d_status, 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e != cudaSuccess || e2 != cudaSuccess) return VOX_CUDA_ECUDA;
    if (*st) {
        uint32_t v = *st;
        cudaMemsetAsync(t->d_status, 0, 4, s);
        cudaStreamSynchronize(s);
        return status_error(v);
    }
    return VOX_CUDA_OK;
}

static int small_rays(const vox_cuda_tree *t, const float *o, const float *d, const uint32_t *roots, size_t n,
                      uint32_t *leaf, uint8_t *slot, float *pts, cudaStream_t s)
{
    HostCallState *hc = host_call_state();
    if (!hc || !small_buffer(hc)) return VOX_CUDA_ENOMEM;
    unsigned char *h = hc->h_small, *dv = hc->d_small;
    std::memcpy(h, o, n * 12);
    std::memcpy(h + SMALL_REGION, d, n * 12);
    if (roots) std::memcpy(h + 2 * SMALL_REGION, roots, n * 4);
    if (pts) std::memcpy(h + 3 * SMALL_REGION, pts, n * 12);   // points are written on hits only
    cudaError_t e = launch_rays<false>(t, reinterpret_cast<const float *>(dv),
                                       reinterpret_cast<const float *>(dv + SMALL_REGION),
                                       roots ? reinterpret_cast<const uint32_t *>(dv + 2 * SMALL_REGION) : nullptr,
                                       n, reinterpret_cast<uint32_t *>(dv + 4 * SMALL_REGION),
                                       dv + 5 * SMALL_REGION,
                                       pts ? reinterpret_cast<float *>(dv + 3 * SMALL_REGION) : nullptr, nullptr, s);
    int rc = small_finish(hc, t, s, e);
    if (rc == VOX_CUDA_ECUDA) return rc;
    std::memcpy(leaf, h + 4 * SMALL_REGION, n * 4);
    if (slot) std::memcpy(slot, h + 5 * SMALL_REGION, n);
    if (pts) std::memcpy(pts, h + 3 * SMALL_REGION, n * 12);
    return rc;
}

static int small_balls(const vox_cuda_tree *t, const float *c, const float *r, size_t n, uint8_t *hit,
                       cudaStream_t s)
{
    HostCallState *hc = host_call_state();
    if (!hc || !small_buffer(hc)) return VOX_CUDA_ENOMEM;
    unsigned char *h = hc->h_small, *dv = hc->d_small;
    std::memcpy(h, c, n * 12);
    std::memcpy(h + SMALL_REGION, r, n * 4);
    cudaError_t e = launch_balls<false>(t, reinterpret_cast<const float *>(dv),
                                        reinterpret_cast<const float *>(dv + SMALL_REGION), n,
                                        dv + 2 * SMALL_REGION, nullptr, s);
    int rc = small_finish(hc, t, s, e);
    if (rc == VOX_CUDA_ECUDA) return rc;
    std::memcpy(hit, h + 2 * SMALL_REGION, n);
    return rc;
}

// The texture on the device for a host-buffer call: uploaded only when its
// bytes differ from the previous call's.
static cudaError_t host_call_texture(HostCallState *hc, const uint8_t *tex, cudaStream_t s)
{
    if (hc->tex_ok && std::memcmp(hc->h_tex, tex, 32768) == 0) return cudaSuccess;
    std::memcpy(hc->h_tex, tex, 32768);
    hc->tex_ok = false;
    cudaError_t e = cudaMemcpyAsync(hc->d_tex, hc->h_tex, 32768, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) hc->tex_ok = true;
    return e;
}

// Ends a host-buffer call: reads the tree's status word back through pinned
// memory with the stream's one synchronisation; clears it if set.  On an
// enqueue error the stream is drained first, so no copy still reads the
// thread's buffers when the call returns.
static int host_call_finish(HostCallState *hc, const vox_cuda_tree *t, cudaStream_t s, cudaError_t e)
{
    if (e == cudaSuccess) e = cudaMemcpyAsync(hc->h_status, t->d_status, 4, cudaMemcpyDeviceToHost, s);
    cudaError_t e2 = cudaStreamSynchronize(s);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        hc->tex_ok = false;
        return VOX_CUDA_ECUDA;
    }
    if (*hc->h_status) {
        cudaMemsetAsync(t->d_status, 0, 4, s);
        cudaStreamSynchronize(s);
        return status_error(*hc->h_status);
    }
    return VOX_CUDA_OK;
}

// The parts of host frame `f` (w x h) outside the traced rectangle r (x0, y0,
// x1, y1; empty: the whole frame), which the finished frame holds as zeros,
// written from the device zero buffer `zero` (at least w * h pixels).
static cudaError_t copy_outside(uint32_t *f, const uint32_t *zero, uint32_t w, uint32_t h, const uint32_t r[4],
                                cudaStream_t cs)
{
    const size_t row = (size_t)w * 4;
    if (r[2] <= r[0] || r[3] <= r[1]) return cudaMemcpyAsync(f, zero, row * h, cudaMemcpyDeviceToHost, cs);
    cudaError_t e = cudaSuccess;
    const uint32_t x0 = r[0], y0 = r[1], x1 = r[2], y1 = r[3], rows = y1 - y0;
    if (y0) e = cudaMemcpyAsync(f, zero, row * y0, cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess && y1 < h)
        e = cudaMemcpyAsync(f + (size_t)y1 * w, zero, row * (h - y1), cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess && x0)
        e = cudaMemcpy2DAsync(f + (size_t)y0 * w, row, zero, (size_t)x0 * 4, (size_t)x0 * 4, rows,
                              cudaMemcpyDeviceToHost, cs);
    if (e == cudaSuccess && x1 < w)
        e = cudaMemcpy2DAsync(f + (size_t)y0 * w + x1, row, zero, (size_t)(w - x1) * 4, (size_t)(w - x1) * 4, rows,
                              cudaMemcpyDeviceToHost, cs);
    return e;
}

// The copy stream, its event and `zeros` bytes of device zeros of the
// calling thread's host calls (grow only; the zeros are written when
// allocated, on stream s, which is then drained, so that no kernel has to run
// before a copy reads them).
static cudaError_t host_call_copies(HostCallState *hc, size_t zeros, cudaStream_t s)
{
    cudaError_t e = cudaSuccess;
    if (!hc->copy) e = cudaStreamCreateWithFlags(&hc->copy, cudaStreamNonBlocking);
    if (e == cudaSuccess && !hc->fin) e = cudaEventCreateWithFlags(&hc->fin, cudaEventDisableTiming);
    if (e == cudaSuccess && hc->zero_bytes < zeros) {
        if (hc->d_zero) {
            cudaDeviceSynchronize();   // an earlier call's copies may still read the old zeros
            cudaFree(hc->d_zero);
            hc->d_zero = nullptr;
            hc->zero_bytes = 0;
        }
        e = cudaMalloc(&hc->d_zero, zeros);
        if (e == cudaSuccess) e = cudaMemsetAsync(hc->d_zero, 0, zeros, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e == cudaSuccess) hc->zero_bytes = zeros;
        else if (hc->d_zero) {
            cudaFree(hc->d_zero);
            hc->d_zero = nullptr;
        }
    }
    return e;
}

// The calling thread's device frame for its single-frame host calls, at
// least `bytes` (grow only; a call returns only after its stream finished
// with it).  Kept rather than taken from the stream-ordered pool each call
// (which returns freed memory at every synchronisation): 1-2.5 us a 1080p
// call.
static uint32_t *host_call_frame(HostCallState *hc, size_t bytes)
{
    if (hc->frame_bytes >= bytes) return hc->d_frame;
    if (hc->d_frame) cudaFree(hc->d_frame);
    hc->d_frame = nullptr;
    hc->frame_bytes = 0;
    void *p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
    hc->d_frame = static_cast<uint32_t *>(p);
    hc->frame_bytes = bytes;
    return hc->d_frame;
}

// A single-frame host call's frame, drawn into device memory at d_argb with
// traced rectangle m, into the host buffer argb: the zeros outside the
// rectangle from the copy stream, which starts at once and runs beside the
// kernel, then the rectangle once the kernel is done (on s, which also waits
// for the zeros).  A 1080p orbit frame, BEST / ADAPTIVE: 140 / 167 us into a
// page-locked frame against 148 / 176 drawn in place over the host link,
// 147 / 175 us into a pageable one against 183 / 211 with the whole frame
// copied after the kernel.
static cudaError_t host_frame_out(HostCallState *hc, uint32_t *argb, const uint32_t *d_argb, uint32_t w, uint32_t h,
                                  const FrameMemo &m, cudaStream_t s)
{
    const size_t npx = (size_t)w * h;
    if (!m.valid) return cudaMemcpyAsync(argb, d_argb, npx * 4, cudaMemcpyDeviceToHost, s);
    const uint32_t r[4] = {m.x0, m.y0, m.x1, m.y1};
    cudaError_t e = copy_outside(argb, hc->d_zero, w, h, r, hc->copy);
    if (e == cudaSuccess) e = cudaEventRecord(hc->fin, hc->copy);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, hc->fin, 0);
    if (e != cudaSuccess) {
        cudaStreamSynchronize(hc->copy);   // no copy may still write argb once the call has returned
        return e;
    }
    if (e == cudaSuccess && r[2] > r[0] && r[3] > r[1]) {
        size_t off = (size_t)r[1] * w + r[0];
        e = cudaMemcpy2DAsync(argb + off, (size_t)w * 4, d_argb + off, (size_t)w * 4, (size_t)(r[2] - r[0]) * 4,
                              r[3] - r[1], cudaMemcpyDeviceToHost, s);
    }
    return e;
}

// Host-buffer frame: the texture is copied in, the frame drawn into device
// scratch and copied out in two parts (host_frame_out).
EXPORT int vox_cuda_render(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                           const uint8_t *tex, uint32_t *argb, void *stream)
try {
    int rc = check_render_args(t, cam, w, h, tex, argb);
    if (rc) return rc;
    cudaStream_t s = as_stream(stream);
    size_t npx = (size_t)w * h;
    HostCallState *hc = host_call_state();
    if (!hc) return VOX_CUDA_ENOMEM;
    if (host_call_copies(hc, npx * 4, s) != cudaSuccess) return VOX_CUDA_ENOMEM;
    uint32_t *d_argb = host_call_frame(hc, npx * 4);
    if (!d_argb) return VOX_CUDA_ENOMEM;
    FrameMemo m{false, 0, 0, 0, 0};
    cudaError_t e = host_call_texture(hc, tex, s);
    if (e == cudaSuccess) e = launch_render<false>(t, *cam, w, h, hc->d_tex, d_argb, nullptr, s, false, nullptr, &m);
    if (e == cudaSuccess) e = host_frame_out(hc, argb, d_argb, w, h, m, s);
    return host_call_finish(hc, t, s, e);
} VOX_ABI_FAIL_INT

// Host-buffer frames of one tree: the texture copied in once; all frames
// drawn by one persistent launch into device frames, one after another, each
// announced when complete; the calling thread waits for each announcement and
// has the frame copied out on a second stream at once, while later frames are
// still drawn; one synchronisation at the end.  Up to STAGE_BYTES of device
// frames (at most 1024 frames) go into one launch; beyond that, launches
// follow one another, reusing the device frames once copied out.
static constexpr size_t STAGE_BYTES = size_t(2) << 30;
static constexpr uint32_t LAUNCH_FRAMES = 1024;
// Frames at the end of a launch sent to the host in two parts (copy_outside
// early, the traced rectangle when drawn): the copy engine moves 184 GB/s to
// host memory, a 1080p frame in 46 us, and the last three or so frames of a
// launch complete within that of each other.  On the 120-frame 1080p orbit
// the call took 7.60 ms with whole-frame copies throughout (the copies
// running 0.15 ms past the kernel's end) and 7.44 ms with this.
static constexpr uint32_t TAIL_FRAMES = 4;


// Waits for flags[j] == epoch; gives up when the stream holding the launch
// has finished or failed without it, or after `limit_s` seconds.
static int wait_announced(const volatile uint32_t *flag, uint32_t epoch, cudaStream_t s, double limit_s)
{
    auto t0 = std::chrono::steady_clock::now();
    for (uint64_t spin = 0;; spin++) {
        if (*flag == epoch) return VOX_CUDA_OK;
        if ((spin & 1023u) == 1023u) {
            cudaError_t q = cudaStreamQuery(s);
            if (q != cudaErrorNotReady) return *flag == epoch ? VOX_CUDA_OK : VOX_CUDA_ECUDA;
            if (std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() > limit_s)
                return VOX_CUDA_ETIMEOUT;
        }
    }
}

EXPORT int vox_cuda_render_frames(const vox_cuda_tree *t, const vox_cuda_camera *cams, uint32_t n, uint32_t w,
                                  uint32_t h, const uint8_t *tex, uint32_t *const *frames, void *stream)
try {
    if (!t || (n && (!cams || !frames))) return VOX_CUDA_EINVAL;
    if (n == 0) return VOX_CUDA_OK;
    for (uint32_t i = 0; i < n; i++) {
        int rc = check_render_args(t, &cams[i], w, h, tex, frames[i]);
        if (rc) return rc;
    }
    int dev = 0, nsm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return VOX_CUDA_ENODEV;
    cudaStream_t s = as_stream(stream);
    size_t npx = (size_t)w * h, fb = npx * 4;
    uint32_t slots = (uint32_t)std::min<size_t>(n, std::max<size_t>(1, STAGE_BYTES / fb));
    uint32_t group = std::min(slots, LAUNCH_FRAMES), ngroups = (n + group - 1) / group;
    size_t tb = align256(frame_job_table_bytes(group));
    HostCallState *hc = host_call_state();
    if (!hc) return VOX_CUDA_ENOMEM;
    cudaError_t e = stage_reserve(hc, slots * fb, slots, ngroups * tb, tb, group, fb, s);
    if (e != cudaSuccess) return e == cudaErrorMemoryAllocation ? VOX_CUDA_ENOMEM : VOX_CUDA_ECUDA;
    std::vector<uint32_t> rects(4 * (size_t)group);
    uint32_t *d_counter = reinterpret_cast<uint32_t *>(static_cast<unsigned char *>(hc->d_table) + tb);
    hc->tex_ok = false;   // copied in by every call: the texture is an input of the frames
    e = host_call_texture(hc, tex, s);
    int rc = VOX_CUDA_OK;
    std::vector<vox_cuda_frame_job> jobs(group);
    for (uint32_t g = 0; g < ngroups && e == cudaSuccess && rc == VOX_CUDA_OK; g++) {
        uint32_t a = g * group, cnt = std::min(group, n - a), epoch = ++hc->epoch;
        for (uint32_t j = 0; j < cnt && e == cudaSuccess; j++) {
            uint32_t i = a + j, b = i % slots;
            if (i >= slots) e = cudaStreamWaitEvent(s, hc->copied[b], 0);   // device frame copied out
            jobs[j] = vox_cuda_frame_job{t, cams[i], w, h, hc->d_tex, hc->d_stage + (size_t)b * npx};
        }
        if (e != cudaSuccess) break;
        rc = enqueue_announced_frames(jobs.data(), cnt, hc->h_tables + (size_t)g * tb, hc->d_table, d_counter,
                                      hc->d_done, hc->d_flags, epoch, nsm, s, rects.data());
        // The launch's last frames complete last, so their copies would follow
        // the kernel's end.  For those, the parts outside the traced rectangle
        // (zeros in the finished frame) go into the host frames now, while the
        // copy stream waits for the first frames anyway, and only the
        // rectangle is copied once the frame is complete.
        // (The copy stream runs copies only: a kernel there, such as a
        // memset, would wait for the persistent kernel to end.)
        uint32_t tail0 = cnt > TAIL_FRAMES ? cnt - TAIL_FRAMES : 0;
        for (uint32_t j = tail0; j < cnt && rc == VOX_CUDA_OK && e == cudaSuccess; j++)
            e = copy_outside(frames[a + j], hc->d_zero, w, h, &rects[4 * (size_t)j], hc->copy);
        for (uint32_t j = 0; j < cnt && rc == VOX_CUDA_OK && e == cudaSuccess; j++) {
            uint32_t i = a + j, b = i % slots;
            rc = wait_announced(hc->h_flags + j, epoch, s, 60.0);
            if (rc) break;
            const uint32_t *r = &rects[4 * (size_t)j];
            const uint32_t *src = hc->d_stage + (size_t)b * npx;
            if (j < tail0)
                e = cudaMemcpyAsync(frames[i], src, fb, cudaMemcpyDeviceToHost, hc->copy);
            else if (r[2] > r[0] && r[3] > r[1]) {
                size_t off = (size_t)r[1] * w + r[0];
                e = cudaMemcpy2DAsync(frames[i] + off, (size_t)w * 4, src + off, (size_t)w * 4,
                                      (size_t)(r[2] - r[0]) * 4, r[3] - r[1], cudaMemcpyDeviceToHost, hc->copy);
            }
            if (e == cudaSuccess) e = cudaEventRecord(hc->copied[b], hc->copy);
        }
    }
    // the call's stream waits for every copy enqueued, so its synchronisation covers them
    cudaError_t e2 = cudaEventRecord(hc->fin, hc->copy);
    if (e2 == cudaSuccess) e2 = cudaStreamWaitEvent(s, hc->fin, 0);
    if (e == cudaSuccess) e = e2;
    int rf = host_call_finish(hc, t, s, e);
    return rc ? rc : rf;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_render_counts_device(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w,
                                         uint32_t h, uint64_t *counts, void *stream)
try {
    if (!t || !cam || !counts) return VOX_CUDA_EINVAL;
    if (w == 0 || h == 0 || (w & 0xF) || (h & 0x3)) return VOX_CUDA_EGEOMETRY;
    return status_of(launch_render<true>(t, *cam, w, h, nullptr, nullptr,
                                         reinterpret_cast<unsigned long long *>(counts), as_stream(stream)));
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_ray_counts_device(const vox_cuda_tree *t, const float *o, const float *d, size_t n,
                                      uint64_t *counts, void *stream)
try {
    if (!t || !counts || (n && (!o || !d))) return VOX_CUDA_EINVAL;
    return status_of(launch_rays<true>(t, o, d, nullptr, n, nullptr, nullptr, nullptr,
                                       reinterpret_cast<unsigned long long *>(counts), as_stream(stream)));
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_ball_counts_device(const vox_cuda_tree *t, const float *c, const float *r, size_t n,
                                       uint64_t *counts, void *stream)
try {
    if (!t || !counts || (n && (!c || !r))) return VOX_CUDA_EINVAL;
    return status_of(launch_balls<true>(t, c, r, n, nullptr,
                                        reinterpret_cast<unsigned long long *>(counts), as_stream(stream)));
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_frame_rect(const float *bbox, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                               uint32_t *rect)
try {
    if (!bbox || !cam || !rect) return VOX_CUDA_EINVAL;
    if (cam->kind != VOX_CUDA_CAMERA_SIMPLE && cam->kind != VOX_CUDA_CAMERA_DOOM) return VOX_CUDA_EINVAL;
    if (w == 0 || h == 0 || (w & 0xF) || (h & 0x3)) return VOX_CUDA_EGEOMETRY;
    double c[2];
    frame_rect(bbox, *cam, w, h, rect, c);
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_render_set_config(const vox_cuda_render_config *cfg)
try {
    if (!cfg || cfg->cull > 1 || cfg->overlap > 1) return VOX_CUDA_EINVAL;
    g_render_cull.store(cfg->cull);
    g_render_overlap.store(cfg->overlap);
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_render_get_config(vox_cuda_render_config *cfg)
try {
    if (!cfg) return VOX_CUDA_EINVAL;
    cfg->cull = g_render_cull.load();
    cfg->overlap = g_render_overlap.load();
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

static bool valid_quality(unsigned int q)
{
    if ((q & VOX_CUDA_QUALITY_RM_MASK) && ((q & VOX_CUDA_QUALITY_MODE_MASK) != VOX_CUDA_QUALITY_ADAPTIVE))
        return false;
    if ((q & VOX_CUDA_QUALITY_MODE_MASK) > VOX_CUDA_QUALITY_ADAPTIVE) return false;
    if ((q & VOX_CUDA_QUALITY_RM_MASK) > VOX_CUDA_QUALITY_RAY_MERGE_ACCURATE) return false;
    return true;
}

// A light manager's snapshot on the device (vox_cuda_lights_upload).
struct vox_cuda_lights {
    float4 *d_nodes = nullptr;
    float4 *d_spheres = nullptr;
    vox::DevLights dev{};
};

int render_frame_memo(const vox_cuda_tree *t, const vox_cuda_camera *cam, const float *dirs, uint32_t w, uint32_t h,
                      unsigned int quality, const uint8_t *tex, const vox_cuda_lights *lights, uint32_t *argb,
                      cudaStream_t s, FrameMemo *memo)
{
    // (a call refused here writes nothing: the memo still holds)
    int rc = check_render_args(t, cam, w, h, tex, argb);
    if (rc) return rc;
    if (!valid_quality(quality)) return VOX_CUDA_EINVAL;
    const vox::DevLights *L = lights ? &lights->dev : nullptr;
    if (!dirs && (quality & VOX_CUDA_QUALITY_MODE_MASK) == VOX_CUDA_QUALITY_BEST)
        return status_of(launch_render<false>(t, *cam, w, h, tex, argb, nullptr, s, true, L, memo));
    return status_of(launch_render_squares(t, *cam, w, h, quality, tex, argb, s, L, dirs, memo));
}

static int render_any_device(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                             unsigned int quality, const uint8_t *tex, const vox_cuda_lights *lights,
                             uint32_t *argb, void *stream)
{
    return render_frame_memo(t, cam, nullptr, w, h, quality, tex, lights, argb, as_stream(stream), nullptr);
}

EXPORT int vox_cuda_render_quality_device(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w,
                                          uint32_t h, unsigned int quality, const uint8_t *tex, uint32_t *argb,
                                          void *stream)
try {
    return render_any_device(t, cam, w, h, quality, tex, nullptr, argb, stream);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_render_lit_device(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                                      unsigned int quality, const uint8_t *tex, const vox_cuda_lights *lights,
                                      uint32_t *argb, void *stream)
try {
    return render_any_device(t, cam, w, h, quality, tex, lights, argb, stream);
} VOX_ABI_FAIL_INT

/* vox_render for a camera class the device cannot compute (renderer.c:200-319
 * with camera->iface->screen2world run by the caller): each pixel's direction
 * is read from `dirs` (device memory, 3 floats a pixel, row by row), all rays
 * start at `origin`.  Every quality is drawn in 4x4 squares as the reference
 * draws them. */
EXPORT int vox_cuda_render_rays_device(const vox_cuda_tree *t, const float *origin, const float *dirs, uint32_t w,
                                       uint32_t h, unsigned int quality, const uint8_t *tex,
                                       const vox_cuda_lights *lights, uint32_t *argb, void *stream)
try {
    if (!origin || !dirs) return VOX_CUDA_EINVAL;
    vox_cuda_camera cam;
    std::memset(&cam, 0, sizeof cam);
    cam.kind = VOX_CUDA_CAMERA_SIMPLE;   // only its position is read
    for (int a = 0; a < 3; a++) cam.position[a] = origin[a];
    return render_frame_memo(t, &cam, dirs, w, h, quality, tex, lights, argb, as_stream(stream), nullptr);
} VOX_ABI_FAIL_INT

static int render_any_host(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                           unsigned int quality, const uint8_t *tex, const vox_cuda_lights *lights, uint32_t *argb,
                           void *stream)
{
    int rc = check_render_args(t, cam, w, h, tex, argb);
    if (rc) return rc;
    if (!valid_quality(quality)) return VOX_CUDA_EINVAL;
    cudaStream_t s = as_stream(stream);
    size_t npx = (size_t)w * h;
    HostCallState *hc = host_call_state();
    if (!hc) return VOX_CUDA_ENOMEM;
    if (host_call_copies(hc, npx * 4, s) != cudaSuccess) return VOX_CUDA_ENOMEM;
    uint32_t *d_argb = host_call_frame(hc, npx * 4);
    if (!d_argb) return VOX_CUDA_ENOMEM;
    cudaError_t e = host_call_texture(hc, tex, s);
    if (e == cudaSuccess) {
        FrameMemo m{false, 0, 0, 0, 0};
        rc = render_frame_memo(t, cam, nullptr, w, h, quality, hc->d_tex, lights, d_argb, s, &m);
        if (rc) {
            host_call_finish(hc, t, s, cudaErrorUnknown);
            return rc;
        }
        e = host_frame_out(hc, argb, d_argb, w, h, m, s);
    }
    return host_call_finish(hc, t, s, e);
}

EXPORT int vox_cuda_render_quality(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                                   unsigned int quality, const uint8_t *tex, uint32_t *argb, void *stream)
try {
    return render_any_host(t, cam, w, h, quality, tex, nullptr, argb, stream);
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_render_lit(const vox_cuda_tree *t, const vox_cuda_camera *cam, uint32_t w, uint32_t h,
                               unsigned int quality, const uint8_t *tex, const vox_cuda_lights *lights, uint32_t *argb,
                               void *stream)
try {
    return render_any_host(t, cam, w, h, quality, tex, lights, argb, stream);
} VOX_ABI_FAIL_INT

// ------------------------------------------------------------------ lights

EXPORT int vox_cuda_lights_upload(const struct vox_light_manager *lm, vox_cuda_lights **out)
try {
    if (!lm || !out) return VOX_CUDA_EINVAL;
    *out = nullptr;
    lights_image img;
    if (lights_flatten(lm, &img)) return VOX_CUDA_ENOMEM;
    // (children - 1) pending records per level fit the search stack
    if (img.depth > 1 + vox::LIGHT_STACK / (VOX_MTREE_MAX_CHILDREN - 1)) {
        lights_image_free(&img);
        return VOX_CUDA_EDEPTH;
    }
    vox_cuda_lights *l = new (std::nothrow) vox_cuda_lights();
    if (!l) { lights_image_free(&img); return VOX_CUDA_ENOMEM; }
    l->dev.ar = img.ambient[0];
    l->dev.ag = img.ambient[1];
    l->dev.ab = img.ambient[2];
    l->dev.on = 1;
    cudaError_t e = cudaSuccess;
    if (img.n_nodes) {
        size_t nb = img.n_nodes * 32, sb = (img.n_spheres ? img.n_spheres : 1) * 32;
        e = cudaMalloc(&l->d_nodes, nb);
        if (e == cudaSuccess) e = cudaMalloc(&l->d_spheres, sb);
        if (e == cudaSuccess) e = cudaMemcpy(l->d_nodes, img.nodes, nb, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemcpy(l->d_spheres, img.spheres, sb, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaStreamSynchronize(cudaStreamLegacy);
        l->dev.nodes = l->d_nodes;
        l->dev.spheres = l->d_spheres;
        l->dev.n_nodes = (uint32_t)img.n_nodes;
        l->dev.n_spheres = (uint32_t)img.n_spheres;
    }
    lights_image_free(&img);
    if (e != cudaSuccess) {
        cudaFree(l->d_nodes);
        cudaFree(l->d_spheres);
        delete l;
        return e == cudaErrorMemoryAllocation ? VOX_CUDA_ENOMEM : VOX_CUDA_ECUDA;
    }
    *out = l;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_lights_free(vox_cuda_lights *l)
try {
    if (!l) return VOX_CUDA_EINVAL;
    cudaFree(l->d_nodes);
    cudaFree(l->d_spheres);
    delete l;
    return VOX_CUDA_OK;
} VOX_ABI_FAIL_INT
