/*
 * raysort.cu -- the order in which a large ray batch is traced.
 *
 * Every ray of a batch is an independent search, so the order in which they
 * are traced changes no result, only how alike the 32 searches of a warp are.
 * Rays given in random order (origins anywhere, directions anywhere) put 32
 * unrelated searches in every warp.  Tracing them grouped by the octant of
 * their direction, then by the cell of the point where they enter the tree's
 * box on an 8x8x8 grid over it (Morton order), makes the searches of a warp
 * start at the same part of the tree and walk it the same way: 16M random
 * rays over the 256^3 tree take 2.8 ms, sorting included, against 5.4 ms in
 * the given order.  Ball batches of 262,144 or more are grouped the same way
 * by the cell of their centre on a 16x16x16 grid over the tree's box: 1M
 * random balls take 0.40 ms, sorting included, against 0.47 ms.
 *
 * The order is a counting sort on those 12-bit keys: per block of up to
 * 65,536 items (fewer for smaller batches, so that every SM gets blocks) a
 * histogram in shared memory, the position of each (key, block) pair from a
 * prefix over blocks and keys, then each item's slot in `order`; the search
 * kernel reads the j-th item of the order from where it was given and writes
 * its result there.  Items of one (key, block) pair land in any order among
 * themselves; that, too, changes no result.
 * (Copying the rays into order instead makes a 16M-ray batch slower: each
 * ray's six floats become scattered partial-sector stores.  Finer keys are
 * slower too: the entry point's cell on a 16^3 grid, 2.84-2.87 ms, and the
 * direction's dominant axis added to the key, 2.99 ms, against 2.77-2.78.)
 */
#include <cuda_runtime.h>

#include <cstdint>

#include "internal.h"

namespace {

constexpr int KEY_BITS = 12;
constexpr uint32_t NKEYS = 1u << KEY_BITS;
constexpr int SORT_THREADS = 1024;

// Items one block keys and places: 65,536 for large batches (256 blocks for
// 16M rays), fewer for smaller ones so that a batch of a million still
// spreads over the SMs (8,192 at least, which keeps the per-block
// histograms small beside the items).
size_t items_per_block(size_t n)
{
    size_t per = (n + 255) / 256;
    per = per < 8192 ? 8192 : (per > 65536 ? 65536 : per);
    return per;
}

struct KeyFrame {
    float lo[3], inv[3];   // cell = floor((p - lo) * inv), clamped to the grid
    float blo[3], bhi[3];  // the tree's box, where the rays' entry points are found
};

// Morton index of point i's cell on a (2^bits)^3 grid.
template <int BITS>
__device__ __forceinline__ uint32_t morton_cell(const float *pt, size_t i, const KeyFrame &f)
{
    constexpr float TOP = (float)((1 << BITS) - 1);
    uint32_t cell[3];
    for (int a = 0; a < 3; a++) {
        float q = (pt[3 * i + a] - f.lo[a]) * f.inv[a];
        cell[a] = q >= TOP ? (uint32_t)TOP : (q > 0.0f ? (uint32_t)q : 0u);   // NaN -> 0
    }
    uint32_t m = 0;
    for (int b = 0; b < BITS; b++)
        for (int a = 0; a < 3; a++) m |= ((cell[a] >> b) & 1u) << (3 * b + a);
    return m;
}

// Direction octant, then the cell, on an 8^3 grid over the tree's box, of
// where the ray enters that box (rays that miss it: the last key).  Rays of
// one key start their searches at the same part of the tree and walk it the
// same way; keyed on the origin's cell instead, a warp's rays of one octant
// still entered the box anywhere (16M rays: 3.94 ms against 2.80).
__device__ __forceinline__ uint32_t ray_key(const float *o, const float *d, size_t i, const KeyFrame &f)
{
    uint32_t oct = (d[3 * i] < 0.0f) | ((d[3 * i + 1] < 0.0f) << 1) | ((d[3 * i + 2] < 0.0f) << 2);
    float t0 = 0.0f, t1 = 3.0e38f;
    for (int a = 0; a < 3; a++) {
        const float inv = 1.0f / d[3 * i + a];
        float ta = (f.blo[a] - o[3 * i + a]) * inv, tb = (f.bhi[a] - o[3 * i + a]) * inv;
        if (ta > tb) { float x = ta; ta = tb; tb = x; }
        t0 = fmaxf(t0, ta);      // NaN (a zero direction inside the slab) keeps the bound
        t1 = fminf(t1, tb);
    }
    if (!(t0 <= t1)) return (oct << 9) | 0x1FFu;
    float p[3];
    for (int a = 0; a < 3; a++) p[a] = o[3 * i + a] + t0 * d[3 * i + a];
    return (oct << 9) | morton_cell<3>(p, 0, f);
}

// Keys of a block's items and the block's histogram (block-major): rays
// (d given) by ray_key, balls (d NULL) by the cell of their centre on a
// 16^3 grid over the tree's box.
__global__ void __launch_bounds__(SORT_THREADS) k_keys(const float *o, const float *d, size_t n, size_t per,
                                                        KeyFrame f, uint16_t *keys, uint32_t *hist)
{
    __shared__ uint32_t h[NKEYS];
    for (uint32_t k = threadIdx.x; k < NKEYS; k += SORT_THREADS) h[k] = 0;
    __syncthreads();
    size_t b0 = (size_t)blockIdx.x * per, b1 = b0 + per < n ? b0 + per : n;
    for (size_t i = b0 + threadIdx.x; i < b1; i += SORT_THREADS) {
        uint32_t k = d ? ray_key(o, d, i, f) : morton_cell<4>(o, i, f);
        keys[i] = (uint16_t)k;
        atomicAdd(&h[k], 1u);
    }
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < NKEYS; k += SORT_THREADS) hist[(size_t)blockIdx.x * NKEYS + k] = h[k];
}

// For every key: its count before each block (in place) and its total.
__global__ void k_key_blocks(uint32_t *hist, uint32_t nblocks, uint32_t *total)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= NKEYS) return;
    uint32_t run = 0;
    for (uint32_t b = 0; b < nblocks; b++) {
        uint32_t c = hist[(size_t)b * NKEYS + k];
        hist[(size_t)b * NKEYS + k] = run;
        run += c;
    }
    total[k] = run;
}

// Exclusive scan of the NKEYS totals in place (one block).
__global__ void __launch_bounds__(1024) k_key_starts(uint32_t *total)
{
    __shared__ uint32_t part[1024];
    constexpr uint32_t PER = NKEYS / 1024;
    uint32_t v[PER], s = 0;
    for (uint32_t j = 0; j < PER; j++) {
        v[j] = total[threadIdx.x * PER + j];
        s += v[j];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1) {   // inclusive scan of the parts
        uint32_t x = threadIdx.x >= off ? part[threadIdx.x - off] : 0u;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (uint32_t j = 0; j < PER; j++) {
        total[threadIdx.x * PER + j] = run;
        run += v[j];
    }
}

// Each ray's slot in the traced order.
__global__ void __launch_bounds__(SORT_THREADS) k_place(const uint16_t *keys, size_t n, size_t per,
                                                         const uint32_t *hist, const uint32_t *start, uint32_t *order)
{
    __shared__ uint32_t base[NKEYS];
    for (uint32_t k = threadIdx.x; k < NKEYS; k += SORT_THREADS)
        base[k] = start[k] + hist[(size_t)blockIdx.x * NKEYS + k];
    __syncthreads();
    size_t b0 = (size_t)blockIdx.x * per, b1 = b0 + per < n ? b0 + per : n;
    for (size_t i = b0 + threadIdx.x; i < b1; i += SORT_THREADS) order[atomicAdd(&base[keys[i]], 1u)] = (uint32_t)i;
}

}  // namespace

static size_t up256(size_t x) { return (x + 255) & ~size_t(255); }

size_t ray_order_bytes(size_t n)
{
    size_t nb = (n + items_per_block(n) - 1) / items_per_block(n);
    return up256(n * 2) + up256(n * 4) + nb * NKEYS * 4 + NKEYS * 4 + 256;
}

// The order of n rays (d given) or balls (d NULL) in `scratch`.
static cudaError_t sort_order(const vox_cuda_tree *t, const float *o, const float *d, size_t n, void *scratch,
                              uint32_t **order, cudaStream_t s)
{
    const size_t per = items_per_block(n), nb = (n + per - 1) / per;
    char *p = static_cast<char *>(scratch);
    uint16_t *keys = reinterpret_cast<uint16_t *>(p);
    p += up256(n * 2);
    *order = reinterpret_cast<uint32_t *>(p);
    p += up256(n * 4);
    uint32_t *hist = reinterpret_cast<uint32_t *>(p);
    uint32_t *total = hist + nb * NKEYS;
    // cells over the tree's box: 8 per axis for rays' entry points, 16 for
    // balls' centres
    const float cells = d ? 8.0f : 16.0f;
    KeyFrame f;
    for (int a = 0; a < 3; a++) {
        f.blo[a] = t->bbox[a];
        f.bhi[a] = t->bbox[3 + a];
        f.lo[a] = t->bbox[a];
        f.inv[a] = cells / fmaxf(t->bbox[3 + a] - t->bbox[a], 1e-30f);
    }
    k_keys<<<(unsigned)nb, SORT_THREADS, 0, s>>>(o, d, n, per, f, keys, hist);
    k_key_blocks<<<NKEYS / 256, 256, 0, s>>>(hist, (uint32_t)nb, total);
    k_key_starts<<<1, 1024, 0, s>>>(total);
    k_place<<<(unsigned)nb, SORT_THREADS, 0, s>>>(keys, n, per, hist, total, *order);
    for (int i = 0; i < 4; i++) count_launch();
    return cudaGetLastError();
}

cudaError_t ray_order(const vox_cuda_tree *t, const float *o, const float *d, size_t n, void *scratch,
                      uint32_t **order, cudaStream_t s)
{
    return sort_order(t, o, d, n, scratch, order, s);
}

cudaError_t ball_order(const vox_cuda_tree *t, const float *centres, size_t n, void *scratch, uint32_t **order,
                       cudaStream_t s)
{
    return sort_order(t, centres, nullptr, n, scratch, order, s);
}
