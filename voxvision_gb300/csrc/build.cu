/*
 * build.cu -- voxtrees octrees built on the GPU, straight into the device
 * image of pool_layout.h: the tree that vox_make_tree builds from a voxel set
 * (tree.c:249-338) and the raw-volume reader of datareader.c:11-85.
 *
 * The tree must be the reference's node for node and voxel for voxel, and two
 * steps of its construction are sequential by definition:
 *
 *  - the subdivision centre is the mean of the node's voxels, summed in float
 *    in the set's current order (find_center, tree.c:125-136), so its
 *    rounding depends on that order;
 *  - the set is split by eight in-place swapping passes, one per octant
 *    (sort_set, tree.c:166-183), which leave the voxels of later octants
 *    permuted; the next level's sums and the leaves' voxel order see that
 *    permutation.
 *
 * Both are computed here in parallel and exactly.
 *
 *  Swapping pass.  In one pass over a range, the claimed voxels (those of
 *  the pass's octant) go to the front in their order.  The others behave as
 *  a queue: an unclaimed voxel joins its tail and each claimed voxel moves
 *  the head to the tail.  So the voxel that ends at position t (t at or past
 *  the claimed count) is found by walking back: if position t held a claimed
 *  voxel, the voxel that ends there is the one that stood at C(t), the
 *  number of claimed positions before t, and so on until an unclaimed
 *  position is reached.  Inside a run of claimed positions every step
 *  subtracts the same number (the unclaimed positions before the run), so a
 *  whole run is crossed in one step.  A prefix count gives C, and the list of
 *  unclaimed positions gives each run's start.
 *
 *  Float sum.  Within one binade, adding d >= 0 to acc = A * 2^e (A an
 *  integer in [2^23, 2^24)) gives (A + q + delta) * 2^e with q = floor(d/2^e)
 *  and delta in {0, 1}, which depends on the fraction of d/2^e and, for an
 *  exact half (rounded to even), on the parity of A + q.  A run of additions
 *  is therefore a map from the parity of A to (increment, new parity): a
 *  two-state machine, and such maps compose associatively.  Chunks of 1024
 *  voxels get their map for each of 12 binades in parallel; one thread per
 *  node then walks its chunks, applying the map of the binade the sum is in,
 *  and adds a chunk voxel by voxel only where the sum leaves its binade
 *  inside the chunk (a dozen times per node) or lies below the precomputed
 *  binades.
 *
 * The rest (bounding boxes, the density test, leaf decisions, children) is
 * per node or per voxel.  The tree is built a level at a time.  Then subtree
 * sizes (bottom up), pre-order ids and image offsets (top down) place every
 * node where the host flattener (flatten.cpp) puts it, and one pass writes the
 * records and the leaves' voxel runs: the image equals the host build followed
 * by vox_cuda_tree_upload, byte for byte.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#include "internal.h"
#include "abi_guard.h"

#define EXPORT extern "C" __attribute__((visibility("default")))

namespace {

constexpr uint32_t NONE = 0xFFFFFFFFu;
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr uint32_t SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr uint32_t BIG = 4096;       // nodes with more voxels sum their coordinates by chunks
constexpr uint32_t SMALL = 512;      // nodes with at most this many voxels are split by one warp
constexpr uint32_t TINY = 32;        // nodes with at most this many voxels get their box from one thread
constexpr uint32_t CHUNK = 1024;     // voxels per chunk
constexpr int CHUNK_THREADS = 128;   // 8 consecutive voxels per thread
constexpr int NBIN = 16;             // binades with a precomputed map per chunk
constexpr uint32_t SAT = 1u << 25;   // map increments saturate here (any >= 2^24 is unusable)
constexpr int MAX_LEVELS = 90;       // deeper trees exceed the traversal stack anyway
constexpr uint64_t MAX_VOXELS = 0x7FFFFFFFull;

enum : uint8_t { K_INNER = 0, K_LEAF = 1, K_DENSE = 2, K_OVER = 3 };

// error bits reported by kernels
constexpr uint32_t ERR_WALK = 1u;       // a swapping-pass walk did not end as it must
constexpr uint32_t ERR_BIG_LEAF = 2u;   // a leaf holds 2^30 voxels or more (record limit)
constexpr uint32_t ERR_LAYOUT = 4u;     // a record or voxel run fell outside the image

inline unsigned grid_for(uint64_t n, unsigned threads) { return (unsigned)((n + threads - 1) / threads); }

// ------------------------------------------------------------------ scan
// Exclusive scan of u32 values v(i), i in [0, m): per-tile sums, a one-block
// scan of the tile sums, then each tile's own scan handed to w(i, excl, v(i)).

__device__ __forceinline__ uint32_t warp_incl_scan(uint32_t x)
{
    int lane = threadIdx.x & 31;
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
        if (lane >= off) x += y;
    }
    return x;
}

template <class V>
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_sums(V v, uint64_t m, uint32_t *tile)
{
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t s = 0;
    for (int j = 0; j < SCAN_ITEMS; j++) {
        uint64_t i = base + (uint64_t)j * SCAN_THREADS + threadIdx.x;
        if (i < m) s += v(i);
    }
    for (int off = 16; off; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < SCAN_THREADS / 32; w++) t += ws[w];
        tile[blockIdx.x] = t;
    }
}

__global__ void __launch_bounds__(1024) k_scan_tiles(uint32_t *a, uint32_t n, uint32_t *total)
{
    __shared__ uint32_t ws[32];
    __shared__ uint32_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (uint32_t base = 0; base < n; base += 1024) {
        uint32_t i = base + threadIdx.x;
        uint32_t x = i < n ? a[i] : 0;
        uint32_t incl = warp_incl_scan(x);
        if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = incl;
        __syncthreads();
        if (threadIdx.x < 32) {
            uint32_t w = ws[threadIdx.x];
            ws[threadIdx.x] = warp_incl_scan(w) - w;
        }
        __syncthreads();
        uint32_t c = carry;
        uint32_t excl = c + ws[threadIdx.x >> 5] + incl - x;
        if (i < n) a[i] = excl;
        __syncthreads();
        if (threadIdx.x == 1023) carry = excl + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

template <class V, class W>
__global__ void __launch_bounds__(SCAN_THREADS) k_tile_apply(V v, W w, uint64_t m, const uint32_t *tile)
{
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    uint32_t run = tile[blockIdx.x];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int j = 0; j < SCAN_ITEMS; j++) {
        uint64_t i = base + (uint64_t)j * SCAN_THREADS + threadIdx.x;
        uint32_t x = i < m ? v(i) : 0;
        uint32_t incl = warp_incl_scan(x);
        if (lane == 31) ws[warp] = incl;
        __syncthreads();
        uint32_t before = 0, tot = 0;
        for (int q = 0; q < SCAN_THREADS / 32; q++) {
            uint32_t t = ws[q];
            before += q < warp ? t : 0u;
            tot += t;
        }
        if (i < m) w(i, run + before + incl - x, x);
        run += tot;
        __syncthreads();
    }
}

template <class V, class W>
void scan(V v, W w, uint64_t m, uint32_t *tile, uint32_t *total, cudaStream_t s)
{
    uint32_t nt = (uint32_t)((m + SCAN_TILE - 1) / SCAN_TILE);
    if (nt == 0) {
        cudaMemsetAsync(total, 0, 4, s);
        return;
    }
    k_tile_sums<<<nt, SCAN_THREADS, 0, s>>>(v, m, tile);
    k_scan_tiles<<<1, 1024, 0, s>>>(tile, nt, total);
    k_tile_apply<<<nt, SCAN_THREADS, 0, s>>>(v, w, m, tile);
    count_launch();
    count_launch();
    count_launch();
}

// ------------------------------------------------------------ level arrays

// The nodes of one level, in position order (children are made in parent
// order, octant order, so their voxel ranges ascend).
struct Level {
    uint32_t m = 0;
    void *mem = nullptr;
    uint32_t *start, *n, *cnt, *first_child, *chunk_base, *sub_nodes, *id, *ustart, *rec;
    unsigned long long *sub_units;
    float *box, *centre;
    int *ehi;
    uint8_t *kind, *mask;
};

template <typename T>
T *carve(char *&p, size_t count)
{
    T *r = reinterpret_cast<T *>(p);
    p += (count * sizeof(T) + 255) & ~size_t(255);
    return r;
}

cudaError_t level_alloc(Level &L, uint32_t m, cudaStream_t s)
{
    size_t mm = m ? m : 1;
    size_t bytes = 0;
    auto add = [&](size_t b) { bytes += (b + 255) & ~size_t(255); };
    add(4 * mm); add(4 * mm); add(32 * mm); add(4 * mm); add(4 * mm); add(4 * mm); add(4 * mm); add(4 * mm);
    add(4 * mm); add(8 * mm); add(24 * mm); add(12 * mm); add(12 * mm); add(mm); add(mm);
    cudaError_t e = cudaMallocAsync(&L.mem, bytes, s);
    if (e != cudaSuccess) { L.mem = nullptr; return e; }
    char *p = static_cast<char *>(L.mem);
    L.m = m;
    L.start = carve<uint32_t>(p, mm);
    L.n = carve<uint32_t>(p, mm);
    L.cnt = carve<uint32_t>(p, 8 * mm);
    L.first_child = carve<uint32_t>(p, mm);
    L.chunk_base = carve<uint32_t>(p, mm);
    L.sub_nodes = carve<uint32_t>(p, mm);
    L.id = carve<uint32_t>(p, mm);
    L.ustart = carve<uint32_t>(p, mm);
    L.rec = carve<uint32_t>(p, mm);
    L.sub_units = carve<unsigned long long>(p, mm);
    L.box = carve<float>(p, 6 * mm);
    L.centre = carve<float>(p, 3 * mm);
    L.ehi = carve<int>(p, 3 * mm);
    L.kind = carve<uint8_t>(p, mm);
    L.mask = carve<uint8_t>(p, mm);
    return cudaMemsetAsync(L.cnt, 0, 32 * mm, s);
}

// -------------------------------------------------------- per-level kernels

__global__ void k_seg_of(const uint32_t *start, const uint32_t *n, uint32_t m, uint64_t N, uint32_t *seg_of)
{
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    if (m == 0 || start[0] > t) {
        seg_of[t] = NONE;
        return;
    }
    uint32_t lo = 0, hi = m;   // the last node starting at or before t is in [lo, hi)
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (start[mid] <= t) lo = mid;
        else hi = mid;
    }
    seg_of[t] = t < (uint64_t)start[lo] + n[lo] ? lo : NONE;
}

struct ChunkCount {
    const uint32_t *n;
    __device__ uint32_t operator()(uint64_t k) const { return n[k] > BIG ? (n[k] + CHUNK - 1) / CHUNK : 0u; }
};
struct StoreExcl {
    uint32_t *out;
    __device__ void operator()(uint64_t i, uint32_t excl, uint32_t) const { out[i] = excl; }
};

// The node of chunk c: the last node whose first chunk is at or before c
// (nodes without chunks share their successor's base).
__device__ __forceinline__ uint32_t chunk_node(const uint32_t *chunk_base, uint32_t m, uint32_t c)
{
    uint32_t lo = 0, hi = m;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (chunk_base[mid] <= c) lo = mid;
        else hi = mid;
    }
    return lo;
}

// First-occurrence extremes: the serial scan of tree.c:138-155 keeps the first
// of equal values (which matters only for -0 against +0), so ties go to the
// lower position.
__device__ __forceinline__ void take_min(float &v, uint32_t &i, float v2, uint32_t i2)
{
    if (v2 < v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}
__device__ __forceinline__ void take_max(float &v, uint32_t &i, float v2, uint32_t i2)
{
    if (v2 > v || (v2 == v && i2 < i)) { v = v2; i = i2; }
}

struct Extremes {
    float mn[3], mx[3];
    uint32_t mni[3], mxi[3];
    __device__ void init()
    {
        for (int a = 0; a < 3; a++) {
            mn[a] = INFINITY; mx[a] = -INFINITY; mni[a] = NONE; mxi[a] = NONE;
        }
    }
    __device__ void add(const float *p, uint32_t t)
    {
        for (int a = 0; a < 3; a++) {
            take_min(mn[a], mni[a], p[a], t);
            take_max(mx[a], mxi[a], p[a], t);
        }
    }
    __device__ void merge(const Extremes &o)
    {
        for (int a = 0; a < 3; a++) {
            take_min(mn[a], mni[a], o.mn[a], o.mni[a]);
            take_max(mx[a], mxi[a], o.mx[a], o.mxi[a]);
        }
    }
    __device__ void warp_merge()
    {
        for (int off = 16; off; off >>= 1) {
            Extremes o;
            for (int a = 0; a < 3; a++) {
                o.mn[a] = __shfl_xor_sync(0xffffffffu, mn[a], off);
                o.mx[a] = __shfl_xor_sync(0xffffffffu, mx[a], off);
                o.mni[a] = __shfl_xor_sync(0xffffffffu, mni[a], off);
                o.mxi[a] = __shfl_xor_sync(0xffffffffu, mxi[a], off);
            }
            merge(o);
        }
    }
};

// Partial extremes of one chunk of a big node.
__global__ void __launch_bounds__(CHUNK_THREADS) k_chunk_box(const float *P, Level L, const uint32_t *total,
                                                            float *cv, uint32_t *ci)
{
    __shared__ Extremes part[CHUNK_THREADS / 32];
    uint32_t c = blockIdx.x;
    if (c >= *total) return;
    uint32_t k = chunk_node(L.chunk_base, L.m, c);
    uint64_t b = (uint64_t)L.start[k] + (uint64_t)(c - L.chunk_base[k]) * CHUNK;
    uint64_t e = min(b + CHUNK, (uint64_t)L.start[k] + L.n[k]);
    Extremes x;
    x.init();
    for (uint64_t t = b + threadIdx.x; t < e; t += CHUNK_THREADS) x.add(P + 3 * t, (uint32_t)t);
    x.warp_merge();
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < CHUNK_THREADS / 32; w++) x.merge(part[w]);
        for (int a = 0; a < 3; a++) {
            cv[6 * c + a] = x.mn[a]; ci[6 * c + a] = x.mni[a];
            cv[6 * c + 3 + a] = x.mx[a]; ci[6 * c + 3 + a] = x.mxi[a];
        }
    }
}

// The box of node k and the top binade its coordinate sums can reach.
__device__ void write_box(const Level &L, uint32_t k, const float *mn, const float *mx, const float *v)
{
    uint32_t nk = L.n[k];
    for (int a = 0; a < 3; a++) {
        L.box[6 * k + a] = mn[a];
        float hi = __fadd_rn(mx[a], v[a]);
        L.box[6 * k + 3 + a] = hi;
        // The float sum of nk values in [0, extent] stays below 2 * nk * extent
        // for any nk this builder accepts (each addition rounds up by at most
        // 2^-24 relative); were it ever higher, its chunks would just be added
        // one voxel at a time.
        double bound = 2.0 * (double)nk * (double)__fsub_rn(hi, mn[a]);
        int ehi = -100000;
        if (bound > 0.0 && bound < 1e38) {
            int ex;
            frexp(bound, &ex);
            ehi = ex - 24;           // bound in [2^(ex-1), 2^ex): its ulp exponent
            if (ehi < -149) ehi = -149;
        }
        L.ehi[3 * k + a] = ehi;
    }
}

// Bounding boxes (calc_bounding_box, tree.c:138-155) of nodes of at most TINY
// voxels: the serial scan itself, one thread per node.
__global__ void k_box_thread(const float *P, Level L, float vx, float vy, float vz)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.m || L.n[k] > TINY) return;
    const float *p = P + 3 * (uint64_t)L.start[k];
    float mn[3] = {p[0], p[1], p[2]}, mx[3] = {p[0], p[1], p[2]};
    for (uint32_t i = 1; i < L.n[k]; i++)
        for (int a = 0; a < 3; a++) {
            float x = p[3 * i + a];
            if (x < mn[a]) mn[a] = x;
            else if (x > mx[a]) mx[a] = x;
        }
    float v[3] = {vx, vy, vz};
    write_box(L, k, mn, mx, v);
}

// The other nodes: a warp per node over its voxels, or over its chunks'
// partial extremes for a big node (listed for the centre kernel).
__global__ void k_box_warp(const float *P, Level L, const float *cv, const uint32_t *ci, float vx, float vy,
                           float vz, uint32_t *big, uint32_t *nbig)
{
    uint32_t k = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lane = threadIdx.x & 31;
    if (k >= L.m) return;
    uint32_t nk = L.n[k];
    if (nk <= TINY) return;
    Extremes x;
    x.init();
    if (nk > BIG) {
        uint32_t nch = (nk + CHUNK - 1) / CHUNK, c0 = L.chunk_base[k];
        for (uint32_t j = lane; j < nch; j += 32) {
            Extremes o;
            uint32_t c = c0 + j;
            for (int a = 0; a < 3; a++) {
                o.mn[a] = cv[6 * c + a]; o.mni[a] = ci[6 * c + a];
                o.mx[a] = cv[6 * c + 3 + a]; o.mxi[a] = ci[6 * c + 3 + a];
            }
            x.merge(o);
        }
    } else {
        uint64_t s = L.start[k];
        for (uint32_t j = lane; j < nk; j += 32) x.add(P + 3 * (s + j), (uint32_t)(s + j));
    }
    x.warp_merge();
    if (lane) return;
    float v[3] = {vx, vy, vz};
    write_box(L, k, x.mn, x.mx, v);
    if (nk > BIG) big[atomicAdd(nbig, 1u)] = k;
}

// ---- the two-state machine of a float sum within one binade

struct Tr {
    uint32_t w0, w1;   // for parity p: increment (bits 0-30) and new parity (bit 31)
};

__device__ __forceinline__ Tr tr_id() { return {0u, 0x80000000u}; }

__device__ __forceinline__ Tr tr_cat(Tr f, Tr g)   // f, then g
{
    uint32_t g0 = (f.w0 >> 31) ? g.w1 : g.w0;
    uint32_t g1 = (f.w1 >> 31) ? g.w1 : g.w0;
    Tr r;
    r.w0 = min((f.w0 & 0x7FFFFFFFu) + (g0 & 0x7FFFFFFFu), SAT) | (g0 & 0x80000000u);
    r.w1 = min((f.w1 & 0x7FFFFFFFu) + (g1 & 0x7FFFFFFFu), SAT) | (g1 & 0x80000000u);
    return r;
}

// Adding d >= 0 to A * 2^e, A in [2^23, 2^24), with round to nearest even.
__device__ __forceinline__ Tr tr_elem(float d, int e)
{
    // d / 2^e by a power-of-two multiply: exact, except that an x below the
    // normal range may round, which leaves it far below one half all the same.
    // Binades whose 2^-e is not a normal float never get a usable map.
    if (e < -126 || e > 126) return {SAT, SAT | 0x80000000u};
    float x = __fmul_rn(d, __int_as_float((127 - e) << 23));
    if (!(x < 33554432.0f)) return {SAT, SAT | 0x80000000u};
    float qf = floorf(x);
    float f = __fsub_rn(x, qf);
    uint32_t q = (uint32_t)qf;
    uint32_t up = f > 0.5f, tie = f == 0.5f;
    uint32_t par0 = q & 1u, par1 = par0 ^ 1u;    // parity of A + q for A even / odd
    uint32_t d0 = up | (tie & par0), d1 = up | (tie & par1);
    return {(q + d0) | ((par0 ^ d0) << 31), (q + d1) | ((par1 ^ d1) << 31)};
}

__device__ __forceinline__ Tr tr_shfl_down(Tr t, int off)
{
    return {__shfl_down_sync(0xffffffffu, t.w0, off), __shfl_down_sync(0xffffffffu, t.w1, off)};
}

// Maps of one chunk of a big node, for the NBIN binades ending at the node's
// top binade, per axis; and whether any of its d is non-zero.
__device__ __forceinline__ size_t map_index(uint64_t maxc, int a, uint32_t c, int bi)
{
    return (((size_t)a * maxc + c) * NBIN + bi) * 2;
}

__global__ void __launch_bounds__(CHUNK_THREADS) k_chunk_maps(const float *P, Level L, const uint32_t *total,
                                                             uint32_t *maps, uint8_t *nz, uint64_t maxc)
{
    __shared__ Tr part[NBIN][3][CHUNK_THREADS / 32];
    __shared__ uint32_t any[3];
    uint32_t c = blockIdx.x;
    if (c >= *total) return;
    if (threadIdx.x < 3) any[threadIdx.x] = 0;
    uint32_t k = chunk_node(L.chunk_base, L.m, c);
    uint64_t b = (uint64_t)L.start[k] + (uint64_t)(c - L.chunk_base[k]) * CHUNK;
    uint64_t e = min(b + CHUNK, (uint64_t)L.start[k] + L.n[k]);
    uint64_t t0 = b + (uint64_t)threadIdx.x * 8;
    float d[8][3];
    uint32_t cnt = t0 < e ? (uint32_t)(e - t0 < 8 ? e - t0 : 8) : 0u;
    uint32_t nzm = 0;
    for (int q = 0; q < 8; q++)
        for (int a = 0; a < 3; a++) {
            d[q][a] = (uint32_t)q < cnt ? __fsub_rn(P[3 * (t0 + q) + a], L.box[6 * k + a]) : 0.0f;
            if (d[q][a] > 0.0f) nzm |= 1u << a;
        }
    __syncthreads();
    for (int a = 0; a < 3; a++)
        if (nzm & (1u << a)) atomicOr(&any[a], 1u);
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int bi = 0; bi < NBIN; bi++)
        for (int a = 0; a < 3; a++) {
            int ee = L.ehi[3 * k + a] - (NBIN - 1) + bi;
            Tr t = tr_id();
            for (uint32_t q = 0; q < cnt; q++) t = tr_cat(t, tr_elem(d[q][a], ee));
            for (int off = 1; off < 32; off <<= 1) {
                Tr u = tr_shfl_down(t, off);
                if ((lane & (2 * off - 1)) == 0) t = tr_cat(t, u);
            }
            if (lane == 0) part[bi][a][warp] = t;
        }
    __syncthreads();
    if (threadIdx.x < NBIN * 3) {
        int bi = threadIdx.x / 3, a = threadIdx.x % 3;
        Tr t = part[bi][a][0];
        for (int w = 1; w < CHUNK_THREADS / 32; w++) t = tr_cat(t, part[bi][a][w]);
        size_t o = map_index(maxc, a, c, bi);
        maps[o] = t.w0;
        maps[o + 1] = t.w1;
    }
    if (threadIdx.x < 3) nz[3 * c + threadIdx.x] = (uint8_t)any[threadIdx.x];
}

// acc plus the d of positions [b, e) in order, by one warp (every lane returns
// the same sum): 128 voxels a step, 4 consecutive ones per lane, added by the
// composed map of the binade acc is in, or one at a time when acc is not a
// normal float or the step would leave its binade.
__device__ float warp_sum(const float *P, uint64_t b, uint64_t e, int a, float mn, float acc)
{
    int lane = threadIdx.x & 31;
    float nx[4];
    for (int j = 0; j < 4; j++) {
        uint64_t t = b + 4 * (uint64_t)lane + j;
        nx[j] = t < e ? P[3 * t + a] : mn;
    }
    for (uint64_t s = b; s < e; s += 128) {
        float d[4];
        for (int j = 0; j < 4; j++) d[j] = __fsub_rn(nx[j], mn);   // past e: +0, which changes no sum
        for (int j = 0; j < 4; j++) {                              // the next step's voxels, in flight meanwhile
            uint64_t t = s + 128 + 4 * (uint64_t)lane + j;
            nx[j] = t < e ? P[3 * t + a] : mn;
        }
        uint32_t bits = __float_as_uint(acc), E = bits >> 23;
        if (E >= 1u && E < 255u) {
            int ee = (int)E - 150;
            Tr t = tr_cat(tr_cat(tr_elem(d[0], ee), tr_elem(d[1], ee)), tr_cat(tr_elem(d[2], ee), tr_elem(d[3], ee)));
            for (int off = 1; off < 32; off <<= 1) {
                Tr u = tr_shfl_down(t, off);
                if ((lane & (2 * off - 1)) == 0) t = tr_cat(t, u);
            }
            uint32_t A = (bits & 0x7FFFFFu) | 0x800000u;
            uint32_t w = __shfl_sync(0xffffffffu, (A & 1u) ? t.w1 : t.w0, 0);
            uint32_t An = A + (w & 0x7FFFFFFFu);
            if (An < (1u << 24)) {
                acc = __uint_as_float((E << 23) | (An & 0x7FFFFFu));
                continue;
            }
        }
        for (int l = 0; l < 32; l++)
            for (int j = 0; j < 4; j++) acc = __fadd_rn(__shfl_sync(0xffffffffu, d[j], l), acc);
    }
    return acc;
}

__device__ __forceinline__ float centre_of(float acc, uint32_t nk, float mn, float v)
{
    float mean = __fadd_rn(__fdiv_rn(acc, __uint2float_rn(nk)), mn);
    return __fmul_rn(ceilf(__fdiv_rn(mean, v)), v);
}

// Node kinds and, for nodes of at most BIG voxels, subdivision centres
// (tree.c:249-275, find_center tree.c:125-136, density test geom.c:157-167);
// a warp per node.
__global__ void k_classify(const float *P, Level L, float vx, float vy, float vz)
{
    uint32_t k = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lane = threadIdx.x & 31;
    if (k >= L.m) return;
    uint32_t nk = L.n[k];
    const float *bx = L.box + 6 * k;
    float s0 = __fsub_rn(bx[3], bx[0]), s1 = __fsub_rn(bx[4], bx[1]), s2 = __fsub_rn(bx[5], bx[2]);
    float bbv = __fmul_rn(__fmul_rn(s0, s1), s2);
    float vv = __fmul_rn(__fmul_rn(vx, vy), vz);
    uint8_t kind = fabsf(__fsub_rn(__fmul_rn(__uint2float_rn(nk), vv), bbv)) < vv ? K_DENSE
                 : (nk <= VOX_MAX_DOTS ? K_LEAF : K_INNER);
    if (lane == 0) L.kind[k] = kind;
    if (kind != K_INNER || nk > BIG) return;
    float v[3] = {vx, vy, vz};
    uint64_t s = L.start[k];
    for (int a = 0; a < 3; a++) {
        float acc = warp_sum(P, s, s + nk, a, bx[a], 0.0f);
        if (lane == 0) L.centre[3 * k + a] = centre_of(acc, nk, bx[a], v[a]);
    }
}

// Centres of big nodes: a warp per (node, axis) walks the node's chunks,
// taking each chunk's map of the binade the sum is in from shared memory.
constexpr int CENTRE_WARPS = 4;
__global__ void __launch_bounds__(CENTRE_WARPS * 32) k_centre_big(const float *P, Level L, const uint32_t *big,
                                                                  const uint32_t *nbig, const uint32_t *maps,
                                                                  const uint8_t *nz, uint64_t maxc, float vx,
                                                                  float vy, float vz)
{
    __shared__ uint32_t sm[CENTRE_WARPS][32 * NBIN * 2];
    __shared__ uint8_t snz[CENTRE_WARPS][32];
    uint32_t w = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
    uint32_t j = w / 3;
    int a = (int)(w % 3);
    if (j >= *nbig) return;
    uint32_t k = big[j];
    if (L.kind[k] != K_INNER) return;
    uint32_t nk = L.n[k], nch = (nk + CHUNK - 1) / CHUNK, c0 = L.chunk_base[k];
    uint64_t s = L.start[k], end = s + nk;
    float mn = L.box[6 * k + a], acc = 0.0f;
    int elo = L.ehi[3 * k + a] - (NBIN - 1);
    for (uint32_t g = 0; g < nch; g += 32) {
        uint32_t cnt = min(32u, nch - g);
        const uint32_t *src = maps + map_index(maxc, a, c0 + g, 0);
        __syncwarp();
        for (uint32_t i = lane; i < cnt * NBIN * 2; i += 32) sm[wb][i] = src[i];
        if ((uint32_t)lane < cnt) snz[wb][lane] = nz[3 * (c0 + g + lane) + a];
        __syncwarp();
        for (uint32_t i = 0; i < cnt; i++) {
            if (acc == 0.0f && !snz[wb][i]) continue;   // all of its d are zero
            uint32_t bits = __float_as_uint(acc), E = bits >> 23;
            int bi = (int)E - 150 - elo;
            if (E >= 1u && E < 255u && bi >= 0 && bi < NBIN) {
                uint32_t A = (bits & 0x7FFFFFu) | 0x800000u;
                uint32_t An = A + (sm[wb][(i * NBIN + bi) * 2 + (A & 1u)] & 0x7FFFFFFFu);
                if (An < (1u << 24)) {
                    acc = __uint_as_float((E << 23) | (An & 0x7FFFFFu));
                    continue;
                }
            }
            uint64_t b = s + (uint64_t)(g + i) * CHUNK;
            acc = warp_sum(P, b, min(b + CHUNK, end), a, mn, acc);
        }
    }
    float v[3] = {vx, vy, vz};
    if (lane == 0) L.centre[3 * k + a] = centre_of(acc, nk, mn, v[a]);
}

// The eight swapping passes (sort_set, tree.c:166-183) of nodes of at most
// SMALL voxels: a warp per node in shared memory, each pass in the parallel
// form of the file's header (ballot prefix counts, the walk back for the rest).
constexpr int PART_WARPS = 4;
__global__ void __launch_bounds__(PART_WARPS * 32) k_partition_warp(Level L, uint32_t *idx, uint8_t *oct,
                                                                     uint32_t *err)
{
    __shared__ uint32_t sidx[PART_WARPS][2][SMALL];
    __shared__ uint8_t soct[PART_WARPS][2][SMALL];
    __shared__ uint16_t sc[PART_WARPS][SMALL], su[PART_WARPS][SMALL];
    uint32_t k = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    uint32_t lane = threadIdx.x & 31, wb = threadIdx.x >> 5;
    if (k >= L.m) return;
    uint32_t nk = L.n[k];
    if (L.kind[k] != K_INNER || nk > SMALL) return;
    uint32_t s0 = L.start[k];
    for (uint32_t i = lane; i < nk; i += 32) {
        sidx[wb][0][i] = idx[s0 + i];
        soct[wb][0][i] = oct[s0 + i];
    }
    __syncwarp();
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t from = 0;
    int cur = 0;
    for (uint32_t o = 0; o < 8; o++) {
        const uint32_t *in_i = sidx[wb][cur];
        const uint8_t *in_o = soct[wb][cur];
        uint32_t *out_i = sidx[wb][cur ^ 1];
        uint8_t *out_o = soct[wb][cur ^ 1];
        for (uint32_t i = lane; i < from; i += 32) {   // claimed by earlier passes
            out_i[i] = in_i[i];
            out_o[i] = in_o[i];
        }
        uint32_t run = 0, urun = 0;
        for (uint32_t base = from; base < nk; base += 32) {
            uint32_t t = base + lane;
            bool in = t < nk;
            uint8_t q = in ? in_o[t] : (uint8_t)0xFF;
            bool cl = in && q == o;
            uint32_t bm = __ballot_sync(0xffffffffu, cl), um = __ballot_sync(0xffffffffu, in && !cl);
            uint32_t crel = run + __popc(bm & lt), urel = urun + __popc(um & lt);
            if (in) {
                sc[wb][t] = (uint16_t)crel;
                if (cl) {
                    out_i[from + crel] = in_i[t];
                    out_o[from + crel] = q;
                } else {
                    su[wb][from + urel] = (uint16_t)t;
                }
            }
            run += __popc(bm);
            urun += __popc(um);
        }
        __syncwarp();
        for (uint32_t t = from + run + lane; t < nk; t += 32) {
            uint32_t s = t;
            for (uint32_t steps = 0; in_o[s] == o; steps++) {
                uint32_t u = (s - from) - sc[wb][s];
                if (u == 0 || steps > SMALL) {
                    atomicOr(err, ERR_WALK);
                    break;
                }
                uint32_t a = su[wb][from + u - 1] + 1u;
                uint32_t back = ((s - a) / u + 1) * u;
                if (a > s || back > s - from) {
                    atomicOr(err, ERR_WALK);
                    break;
                }
                s -= back;
            }
            out_i[t] = in_i[s];
            out_o[t] = in_o[s];
        }
        if (lane == 0) L.cnt[8 * k + o] = run;
        from += run;
        cur ^= 1;
        __syncwarp();
    }
    for (uint32_t i = lane; i < nk; i += 32) {   // eight passes: back in buffer 0
        idx[s0 + i] = sidx[wb][0][i];
        oct[s0 + i] = soct[wb][0][i];
    }
}

// Identity permutation and octants (get_subspace_idx, geom.c:44-51) of the
// voxels of nodes to split; 0xFF elsewhere.
__global__ void k_oct_init(const float *P, Level L, const uint32_t *seg_of, uint64_t N, uint32_t *idx, uint8_t *oct)
{
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    idx[t] = (uint32_t)t;
    uint32_t k = seg_of[t];
    if (k == NONE || L.kind[k] != K_INNER) {
        oct[t] = 0xFF;
        return;
    }
    const float *c = L.centre + 3 * k, *p = P + 3 * t;
    oct[t] = (uint8_t)((c[0] > p[0]) | ((c[1] > p[1]) << 1) | ((c[2] > p[2]) << 2));
}

// ---- one swapping pass (sort_set, tree.c:166-183) over every node above SMALL
//
// Four kernels a pass: claimed counts per tile of SCAN_TILE positions (and,
// for every range starting in a tile, the count before its start), a scan of
// the tile counts, the claimed voxels to the front (with each position's
// claimed count since its range start and the unclaimed positions listed),
// then the walk back for the rest of each range.

struct Pass {
    const uint32_t *seg_of, *start, *n, *cnt;
    const uint8_t *kind;
    uint32_t o;
    // The node of position t and where its pass range starts; false when t
    // is outside every pass range (voxels of other octants already claimed,
    // nodes not split here, voxels already in leaves).
    __device__ __forceinline__ bool range(uint64_t t, uint32_t &k, uint32_t &from) const
    {
        k = seg_of[t];
        if (k == NONE || kind[k] != K_INNER || n[k] <= SMALL) return false;
        uint32_t f = start[k];
        for (uint32_t q = 0; q < o; q++) f += cnt[8 * k + q];
        from = f;
        return t >= f;
    }
};

// Block-wide exclusive scan of one flag per thread; *total gets the block's sum.
__device__ __forceinline__ uint32_t block_excl(uint32_t x, uint32_t *ws, uint32_t &total)
{
    int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = warp_incl_scan(x);
    if (lane == 31) ws[warp] = incl;
    __syncthreads();
    uint32_t before = 0, tot = 0;
    for (int q = 0; q < SCAN_THREADS / 32; q++) {
        uint32_t t = ws[q];
        before += q < warp ? t : 0u;
        tot += t;
    }
    __syncthreads();
    total = tot;
    return before + incl - x;
}

// Claimed count of each tile, and for every range starting in the tile the
// count before its start within the tile.
__device__ __forceinline__ void tile_count(const Pass &p, uint64_t t, bool cl, bool head, uint32_t k,
                                           uint32_t &run, uint32_t *ws, uint32_t *head_before)
{
    uint32_t tot;
    uint32_t ex = block_excl(cl ? 1u : 0u, ws, tot);
    if (head) head_before[k] = run + ex;
    run += tot;
}

__global__ void __launch_bounds__(SCAN_THREADS) k_pass_count(Pass p, const uint8_t *oct, uint64_t N,
                                                             uint32_t *tile, uint32_t *head_before)
{
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t run = 0;
    for (int j = 0; j < SCAN_ITEMS; j++) {
        uint64_t t = base + (uint64_t)j * SCAN_THREADS + threadIdx.x;
        uint32_t k = 0, from = 0;
        bool in = t < N && p.range(t, k, from);
        tile_count(p, t, in && oct[t] == p.o, in && t == from, k, run, ws, head_before);
    }
    if (threadIdx.x == 0) tile[blockIdx.x] = run;
}

// Claimed voxels to the front of their range, in order; each position's
// claimed count since its range start (C); unclaimed positions listed; each
// node's claimed count.  Positions outside the ranges are carried over.
__global__ void __launch_bounds__(SCAN_THREADS) k_pass_front(Pass p, uint64_t N, const uint32_t *tile,
                                                             const uint32_t *head_before, const uint8_t *in_oct,
                                                             const uint32_t *in_idx, uint8_t *out_oct,
                                                             uint32_t *out_idx, uint32_t *C, uint32_t *upos,
                                                             uint32_t *cnt)
{
    __shared__ uint32_t ws[SCAN_THREADS / 32];
    uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
    uint32_t run = tile[blockIdx.x];   // claimed positions before this tile
    for (int j = 0; j < SCAN_ITEMS; j++) {
        uint64_t t = base + (uint64_t)j * SCAN_THREADS + threadIdx.x;
        uint32_t k = 0, from = 0;
        bool in = t < N && p.range(t, k, from);
        uint8_t q = t < N ? in_oct[t] : (uint8_t)0xFF;
        bool cl = in && q == p.o;
        uint32_t tot;
        uint32_t ex = block_excl(cl ? 1u : 0u, ws, tot);
        if (t < N) {
            if (!in) {
                out_idx[t] = in_idx[t];
                out_oct[t] = q;
            } else {
                uint32_t cf = tile[from / SCAN_TILE] + head_before[k];   // claimed positions before the range
                uint32_t crel = run + ex - cf;
                C[t] = crel;
                if (cl) {
                    out_idx[from + crel] = in_idx[t];
                    out_oct[from + crel] = q;
                } else {
                    upos[from + ((uint32_t)t - from) - crel] = (uint32_t)t;
                }
                if (t + 1 == (uint64_t)p.start[k] + p.n[k]) cnt[8 * k + p.o] = crel + (cl ? 1u : 0u);
            }
        }
        run += tot;
    }
}

// The rest of each range: the walk back described at the top of the file.
__global__ void k_pass_back(Pass p, uint64_t N, const uint32_t *C, const uint32_t *upos, const uint8_t *in_oct,
                            const uint32_t *in_idx, uint8_t *out_oct, uint32_t *out_idx, uint32_t *err)
{
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    uint32_t k, from;
    if (!p.range(t, k, from) || (uint32_t)t - from < p.cnt[8 * k + p.o]) return;
    uint32_t s = (uint32_t)t;
    for (uint32_t steps = 0; in_oct[s] == p.o; steps++) {
        uint32_t u = (s - from) - C[s];           // unclaimed positions before s
        if (u == 0 || steps > (1u << 22)) {        // impossible for a consistent pass
            atomicOr(err, ERR_WALK);
            break;
        }
        uint32_t a = upos[from + u - 1] + 1;      // start of the claimed run holding s
        uint32_t back = ((s - a) / u + 1) * u;
        if (a > s || back > s - from) {
            atomicOr(err, ERR_WALK);
            break;
        }
        s -= back;
    }
    out_idx[t] = in_idx[s];
    out_oct[t] = in_oct[s];
}

__global__ void k_gather(uint64_t N, const uint32_t *idx, const float *P, float *Pn)
{
    uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= N) return;
    uint64_t i = idx[t];
    Pn[3 * t] = P[3 * i];
    Pn[3 * t + 1] = P[3 * i + 1];
    Pn[3 * t + 2] = P[3 * i + 2];
}

// Overflowed leaves (one octant took the whole set, tree.c:281-305), child
// masks, per-level counts (inner, leaves, dense leaves, leaf voxels) and the
// largest child.
__global__ void k_finish(Level L, unsigned long long *stats, uint32_t *largest, uint32_t *err)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.m) return;
    uint8_t kind = L.kind[k];
    uint32_t mask = 0, top = 0;
    if (kind == K_INNER) {
        bool over = false;
        for (int o = 0; o < 8; o++) {
            uint32_t c = L.cnt[8 * k + o];
            over |= c == L.n[k];
            mask |= (c ? 1u : 0u) << o;
            top = max(top, c);
        }
        if (over) {
            kind = K_OVER;
            mask = 0;
            L.kind[k] = K_OVER;
        } else {
            atomicMax(largest, top);
        }
    }
    L.mask[k] = (uint8_t)mask;
    if (kind == K_INNER) {
        atomicAdd(&stats[0], 1ull);
    } else if (kind == K_DENSE) {
        atomicAdd(&stats[2], 1ull);
    } else {
        atomicAdd(&stats[1], 1ull);
        atomicAdd(&stats[3], (unsigned long long)L.n[k]);
        if (L.n[k] >= (1u << 30)) atomicOr(err, ERR_BIG_LEAF);
    }
}

struct ChildCount {
    const uint8_t *mask;
    __device__ uint32_t operator()(uint64_t k) const { return (uint32_t)__popc(mask[k]); }
};

__global__ void k_children(Level L, Level Nx)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.m || !L.mask[k]) return;
    uint32_t f = L.first_child[k], s = L.start[k];
    for (int o = 0; o < 8; o++) {
        uint32_t c = L.cnt[8 * k + o];
        if (c) {
            Nx.start[f] = s;
            Nx.n[f] = c;
            f++;
        }
        s += c;
    }
}

// ------------------------------------------------------------------ layout

// Units a node appends to the image (its child block or voxel run), nodes and
// units of its subtree (flatten.cpp's placement).
__global__ void k_up(Level L, Level Nx, bool has_next)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.m) return;
    uint8_t kind = L.kind[k];
    uint32_t nch = (uint32_t)__popc(L.mask[k]);
    unsigned long long app = kind == K_INNER ? 3ull * nch : (kind == K_DENSE ? 0ull : L.n[k]);
    uint32_t sn = 1;
    unsigned long long su = app;
    if (kind == K_INNER && has_next) {
        uint32_t f = L.first_child[k];
        for (uint32_t j = 0; j < nch; j++) {
            sn += Nx.sub_nodes[f + j];
            su += Nx.sub_units[f + j];
        }
    }
    L.sub_nodes[k] = sn;
    L.sub_units[k] = su;
}

__global__ void k_root(Level L)
{
    L.id[0] = 0;
    L.rec[0] = 0;
    L.ustart[0] = VOXP_REC_UNITS;
}

// Pre-order ids and image offsets of the children of every inner node.
__global__ void k_down(Level L, Level Nx)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.m || L.kind[k] != K_INNER) return;
    uint32_t nch = (uint32_t)__popc(L.mask[k]);
    uint32_t f = L.first_child[k], us = L.ustart[k];
    uint32_t cid = L.id[k] + 1, cu = us + VOXP_REC_UNITS * nch;
    for (uint32_t j = 0; j < nch; j++) {
        Nx.id[f + j] = cid;
        Nx.ustart[f + j] = cu;
        Nx.rec[f + j] = us + VOXP_REC_UNITS * j;
        cid += Nx.sub_nodes[f + j];
        cu += (uint32_t)Nx.sub_units[f + j];
    }
}

// Node records (pool_layout.h) and the pre-order id map.
__global__ void k_emit(Level L, uint4 *pool, uint32_t *rec_of_id, uint64_t units, uint64_t nodes, uint32_t *err,
                       uint32_t *dots_of_id)
{
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= L.m) return;
    uint8_t kind = L.kind[k];
    uint32_t id = L.id[k], rec = L.rec[k], meta, link;
    if ((uint64_t)rec + VOXP_REC_UNITS > units || id >= nodes) {   // cannot happen for a consistent layout
        atomicOr(err, ERR_LAYOUT);
        return;
    }
    if (dots_of_id) dots_of_id[id] = L.n[k];   // the node's dots_num (tree.c:262)
    uint4 extra = make_uint4(0u, 0u, 0u, 0u);
    if (kind == K_DENSE) {
        meta = VOXP_KIND_DENSE;
        link = id;
    } else if (kind == K_INNER) {
        meta = VOXP_KIND_INNER | ((uint32_t)L.mask[k] << 8);
        link = L.ustart[k];
        const float *c = L.centre + 3 * k;
        extra = make_uint4(__float_as_uint(c[0]), __float_as_uint(c[1]), __float_as_uint(c[2]), 0u);
    } else {
        uint32_t cnt = L.n[k];
        meta = VOXP_KIND_LEAF | (cnt << 2);
        link = L.ustart[k];
        extra = make_uint4(id, cnt, 0u, 0u);
    }
    const float *b = L.box + 6 * k;
    pool[rec] = make_uint4(__float_as_uint(b[0]), __float_as_uint(b[1]), __float_as_uint(b[2]), __float_as_uint(b[3]));
    pool[rec + 1] = make_uint4(__float_as_uint(b[4]), __float_as_uint(b[5]), meta, link);
    pool[rec + 2] = extra;
    rec_of_id[id] = rec;
}

// Voxel runs of the leaves, a warp per node.
__global__ void k_emit_voxels(Level L, const float *P, uint4 *pool, uint64_t units, uint32_t *err)
{
    uint32_t k = (uint32_t)(((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    int lane = threadIdx.x & 31;
    if (k >= L.m) return;
    uint8_t kind = L.kind[k];
    if (kind != K_LEAF && kind != K_OVER) return;
    uint64_t s = L.start[k];
    uint32_t u = L.ustart[k], nk = L.n[k];
    if ((uint64_t)u + nk > units) {
        if (lane == 0) atomicOr(err, ERR_LAYOUT);
        return;
    }
    for (uint32_t i = lane; i < nk; i += 32) {
        const float *p = P + 3 * (s + i);
        pool[u + i] = make_uint4(__float_as_uint(p[0]), __float_as_uint(p[1]), __float_as_uint(p[2]), 0u);
    }
}

// ------------------------------------------------------------ raw reader

struct RawSolid {
    const uint8_t *samples, *mask;
    uint32_t ss, lo, hi;
    __device__ uint32_t operator()(uint64_t v) const
    {
        uint32_t x = 0;
        for (uint32_t l = 0; l < ss; l++) x |= (uint32_t)samples[v * ss + l] << (8 * l);   // datareader.c:61-72
        if (mask) return (mask[x >> 3] >> (x & 7)) & 1u;
        return x >= lo && x <= hi;
    }
};

struct RawPlace {
    uint32_t d1, d2;
    float v0, v1, v2;
    float *P;
    __device__ void operator()(uint64_t v, uint32_t excl, uint32_t solid) const
    {
        if (!solid) return;
        uint64_t jk = (uint64_t)d1 * d2;
        uint32_t i = (uint32_t)(v / jk), j = (uint32_t)((v / d2) % d1), k = (uint32_t)(v % d2);
        // array[counter][a] = index * vox_voxel[a] (datareader.c:73-77)
        P[3 * (uint64_t)excl] = __fmul_rn(__uint2float_rn(i), v0);
        P[3 * (uint64_t)excl + 1] = __fmul_rn(__uint2float_rn(j), v1);
        P[3 * (uint64_t)excl + 2] = __fmul_rn(__uint2float_rn(k), v2);
    }
};

// ---------------------------------------------------------------- host side

struct Dev {
    cudaStream_t s;
    std::vector<void *> owned;
    explicit Dev(cudaStream_t st) : s(st) {}
    template <typename T>
    cudaError_t get(T **p, size_t count)
    {
        void *q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, count * sizeof(T) + 16, s);
        if (e == cudaSuccess) owned.push_back(q);
        *p = static_cast<T *>(q);
        return e;
    }
    ~Dev()
    {
        for (void *p : owned) cudaFreeAsync(p, s);
        cudaStreamSynchronize(s);
    }
};

int fail(cudaError_t e) { return e == cudaErrorMemoryAllocation ? VOX_CUDA_ENOMEM : VOX_CUDA_ECUDA; }

#define TRY(x)                                   \
    do {                                         \
        cudaError_t e_ = (x);                    \
        if (e_ != cudaSuccess) return fail(e_);  \
    } while (0)

// Builds the tree of the N voxels at d_set (device, 3N floats, not modified)
// into t.  Synchronous on s.  With `x`, also hands back what a host tree
// needs beyond the image (see HostTreeExtras).
int build_tree(vox_cuda_tree *t, const float *d_set, uint64_t N, cudaStream_t s, HostTreeExtras *x = nullptr)
{
    const float vx = vox_voxel[0], vy = vox_voxel[1], vz = vox_voxel[2];
    ImageStats st{};
    st.voxel[0] = vx; st.voxel[1] = vy; st.voxel[2] = vz;
    if (N == 0) return adopt_image(t, nullptr, 0, nullptr, 0, st);
    if (N > MAX_VOXELS) return VOX_CUDA_ETOOBIG;

    Dev d(s);
    std::vector<Level> levels;
    struct LevelFree {
        std::vector<Level> &v;
        cudaStream_t s;
        ~LevelFree()
        {
            for (auto &L : v)
                if (L.mem) cudaFreeAsync(L.mem, s);
        }
    } level_free{levels, s};

    float *P[2];
    uint32_t *idx[2], *C, *upos, *seg_of, *tile, *scal, *maps, *cidx, *big;
    uint8_t *oct[2], *nz;
    float *cv;
    unsigned long long *stats;
    uint64_t max_chunks = N / CHUNK + N / BIG + 2;
    uint64_t max_big = N / BIG + 1;
    uint64_t max_tiles = N / SCAN_TILE + 2;
    TRY(d.get(&P[0], 3 * N));
    TRY(d.get(&P[1], 3 * N));
    TRY(d.get(&idx[0], N));
    TRY(d.get(&idx[1], N));
    TRY(d.get(&oct[0], N));
    TRY(d.get(&oct[1], N));
    TRY(d.get(&C, N));
    TRY(d.get(&upos, N));
    TRY(d.get(&seg_of, N));
    TRY(d.get(&tile, max_tiles));
    uint32_t *hbefore;   // per node: claimed count before its range start within its tile
    TRY(d.get(&hbefore, N));
    // scal: 0 chunks, 1 claimed, 2 children, 3 big nodes, 4 largest child, 7 error bits
    TRY(d.get(&scal, 8));
    TRY(d.get(&big, max_big));
    if (N > BIG) {
        TRY(d.get(&cv, 6 * max_chunks));
        TRY(d.get(&cidx, 6 * max_chunks));
        TRY(d.get(&maps, max_chunks * NBIN * 3 * 2));
        TRY(d.get(&nz, 3 * max_chunks));
    } else {
        cv = nullptr;
        cidx = maps = nullptr;
        nz = nullptr;
    }
    TRY(d.get(&stats, 4 * MAX_LEVELS));
    uint32_t *err = scal + 7;
    TRY(cudaMemsetAsync(scal, 0, 8 * 4, s));
    TRY(cudaMemsetAsync(stats, 0, 4 * MAX_LEVELS * sizeof(unsigned long long), s));
    TRY(cudaMemcpyAsync(P[0], d_set, 12 * N, cudaMemcpyDeviceToDevice, s));

    Level root;
    TRY(level_alloc(root, 1, s));
    levels.push_back(root);
    uint32_t root_sn[2] = {0u, (uint32_t)N};
    TRY(cudaMemcpyAsync(levels[0].start, &root_sn[0], 4, cudaMemcpyHostToDevice, s));
    TRY(cudaMemcpyAsync(levels[0].n, &root_sn[1], 4, cudaMemcpyHostToDevice, s));

    const unsigned TB = 256;
    int cur = 0;
    uint32_t *h_next = nullptr;
    TRY(cudaMallocHost(&h_next, 64));
    struct HostFree {
        void *p;
        ~HostFree() { cudaFreeHost(p); }
    } host_free{h_next};

    uint32_t largest = (uint32_t)N;   // the largest node of the level
    for (int lv = 0;; lv++) {
        if (lv >= MAX_LEVELS) return VOX_CUDA_EDEPTH;
        Level L = levels[lv];
        uint32_t m = L.m;
        TRY(cudaMemsetAsync(scal, 0, 5 * 4, s));
        k_seg_of<<<grid_for(N, TB), TB, 0, s>>>(L.start, L.n, m, N, seg_of);
        count_launch();
        bool has_big = largest > BIG;
        if (has_big) {   // chunk extremes of big nodes
            scan(ChunkCount{L.n}, StoreExcl{L.chunk_base}, m, tile, scal + 0, s);
            k_chunk_box<<<(unsigned)max_chunks, CHUNK_THREADS, 0, s>>>(P[cur], L, scal + 0, cv, cidx);
            count_launch();
        }
        k_box_thread<<<grid_for(m, TB), TB, 0, s>>>(P[cur], L, vx, vy, vz);
        count_launch();
        if (largest > TINY) {
            k_box_warp<<<grid_for((uint64_t)m * 32, TB), TB, 0, s>>>(P[cur], L, cv, cidx, vx, vy, vz, big, scal + 3);
            count_launch();
        }
        if (has_big) {
            k_chunk_maps<<<(unsigned)max_chunks, CHUNK_THREADS, 0, s>>>(P[cur], L, scal + 0, maps, nz, max_chunks);
            count_launch();
        }
        k_classify<<<grid_for((uint64_t)m * 32, TB), TB, 0, s>>>(P[cur], L, vx, vy, vz);
        count_launch();
        if (has_big) {
            k_centre_big<<<grid_for(max_big * 3 * 32, CENTRE_WARPS * 32), CENTRE_WARPS * 32, 0, s>>>(
                P[cur], L, big, scal + 3, maps, nz, max_chunks, vx, vy, vz);
            count_launch();
        }
        k_oct_init<<<grid_for(N, TB), TB, 0, s>>>(P[cur], L, seg_of, N, idx[0], oct[0]);
        count_launch();
        if (largest > SMALL) {
            // the eight swapping passes of nodes above SMALL; the result lands back in buffer 0
            unsigned nt = (unsigned)((N + SCAN_TILE - 1) / SCAN_TILE);
            for (uint32_t o = 0; o < 8; o++) {
                int in = o & 1, out = in ^ 1;
                Pass p{seg_of, L.start, L.n, L.cnt, L.kind, o};
                k_pass_count<<<nt, SCAN_THREADS, 0, s>>>(p, oct[in], N, tile, hbefore);
                k_scan_tiles<<<1, 1024, 0, s>>>(tile, nt, scal + 1);
                k_pass_front<<<nt, SCAN_THREADS, 0, s>>>(p, N, tile, hbefore, oct[in], idx[in], oct[out], idx[out], C,
                                                         upos, L.cnt);
                k_pass_back<<<grid_for(N, TB), TB, 0, s>>>(p, N, C, upos, oct[in], idx[in], oct[out], idx[out], err);
                for (int i = 0; i < 4; i++) count_launch();
            }
        }
        k_partition_warp<<<grid_for((uint64_t)m * 32, PART_WARPS * 32), PART_WARPS * 32, 0, s>>>(L, idx[0], oct[0],
                                                                                              err);
        k_gather<<<grid_for(N, TB), TB, 0, s>>>(N, idx[0], P[cur], P[cur ^ 1]);
        cur ^= 1;
        k_finish<<<grid_for(m, TB), TB, 0, s>>>(L, stats + 4 * lv, scal + 4, err);
        count_launch();
        count_launch();
        count_launch();
        scan(ChildCount{L.mask}, StoreExcl{L.first_child}, m, tile, scal + 2, s);
        TRY(cudaGetLastError());
        TRY(cudaMemcpyAsync(h_next, scal + 2, 12, cudaMemcpyDeviceToHost, s));
        TRY(cudaStreamSynchronize(s));
        uint32_t mn = h_next[0];
        largest = h_next[2];
        if (mn == 0) break;
        Level Nx;
        TRY(level_alloc(Nx, mn, s));
        levels.push_back(Nx);
        k_children<<<grid_for(m, TB), TB, 0, s>>>(L, Nx);
        count_launch();
    }

    // bottom up: subtree sizes
    int nl = (int)levels.size();
    for (int lv = nl - 1; lv >= 0; lv--) {
        Level L = levels[lv];
        Level Nx = lv + 1 < nl ? levels[lv + 1] : L;
        k_up<<<grid_for(L.m, 256), 256, 0, s>>>(L, Nx, lv + 1 < nl);
        count_launch();
    }
    std::vector<unsigned long long> h_stats(4 * MAX_LEVELS);
    uint32_t h_root[2];
    unsigned long long h_units = 0;
    float h_box[6];
    TRY(cudaMemcpyAsync(h_stats.data(), stats, 4 * MAX_LEVELS * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                        s));
    TRY(cudaMemcpyAsync(&h_root[0], levels[0].sub_nodes, 4, cudaMemcpyDeviceToHost, s));
    TRY(cudaMemcpyAsync(&h_root[1], err, 4, cudaMemcpyDeviceToHost, s));
    TRY(cudaMemcpyAsync(&h_units, levels[0].sub_units, 8, cudaMemcpyDeviceToHost, s));
    TRY(cudaMemcpyAsync(h_box, levels[0].box, 24, cudaMemcpyDeviceToHost, s));
    TRY(cudaStreamSynchronize(s));
    if (h_root[1] & ERR_WALK) return VOX_CUDA_ECUDA;
    if (h_root[1] & ERR_BIG_LEAF) return VOX_CUDA_ETOOBIG;
    uint64_t units = VOXP_REC_UNITS + h_units;
    if (units > VOXP_MAX_UNITS) return VOX_CUDA_ETOOBIG;
    uint64_t nodes = h_root[0];

    // top down: ids and offsets
    k_root<<<1, 1, 0, s>>>(levels[0]);
    count_launch();
    for (int lv = 0; lv + 1 < nl; lv++) {
        k_down<<<grid_for(levels[lv].m, 256), 256, 0, s>>>(levels[lv], levels[lv + 1]);
        count_launch();
    }
    uint4 *pool = nullptr;
    uint32_t *map = nullptr, *dots = nullptr;
    size_t pool_bytes = units * 16, map_bytes = nodes * 4;
    if (x) TRY(d.get(&dots, nodes));
    TRY(cudaMalloc(&pool, pool_bytes));
    if (cudaMalloc(&map, map_bytes) != cudaSuccess) {
        cudaFree(pool);
        return VOX_CUDA_ENOMEM;
    }
    for (int lv = 0; lv < nl; lv++) {
        Level L = levels[lv];
        k_emit<<<grid_for(L.m, 256), 256, 0, s>>>(L, pool, map, units, nodes, err, dots);
        k_emit_voxels<<<grid_for((uint64_t)L.m * 32, 256), 256, 0, s>>>(L, P[cur], pool, units, err);
        count_launch();
        count_launch();
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_root[1], err, 4, cudaMemcpyDeviceToHost, s);
    if (x) {
        x->dots_of_id.resize(nodes);
        if (e == cudaSuccess && x->order)
            e = cudaMemcpyAsync(x->order, P[cur], 12 * N, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(x->dots_of_id.data(), dots, nodes * 4, cudaMemcpyDeviceToHost, s);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess || h_root[1]) {
        cudaFree(pool);
        cudaFree(map);
        return e != cudaSuccess ? fail(e) : VOX_CUDA_ECUDA;
    }
    st.nodes = nodes;
    st.units = units;
    for (int lv = 0; lv < nl; lv++) {
        st.inner += h_stats[4 * lv];
        st.leaf += h_stats[4 * lv + 1];
        st.dense += h_stats[4 * lv + 2];
        st.dots += h_stats[4 * lv + 3];
        if (h_stats[4 * lv]) st.depth = (uint64_t)lv + 1;
    }
    for (int i = 0; i < 6; i++) st.bbox[i] = h_box[i];
    int rc = adopt_image(t, pool, pool_bytes, map, map_bytes, st);
    if (rc) {
        cudaFree(pool);
        cudaFree(map);
    }
    return rc;
}

struct Stream {
    cudaStream_t s = nullptr;
    Stream() { cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking); }
    ~Stream()
    {
        if (s) cudaStreamDestroy(s);
    }
};

// A new tree handle built by f(t, stream).
template <class F>
int new_tree(vox_cuda_tree **out, F f)
{
    if (!out) return VOX_CUDA_EINVAL;
    *out = nullptr;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return VOX_CUDA_ENODEV;
    Stream st;
    if (!st.s) return VOX_CUDA_ECUDA;
    vox_cuda_tree *t = new (std::nothrow) vox_cuda_tree();
    if (!t) return VOX_CUDA_ENOMEM;
    t->device = dev;
    int rc = f(t, st.s);
    if (rc) {
        vox_cuda_tree_free(t);
        return rc;
    }
    *out = t;
    return VOX_CUDA_OK;
}

int raw_build(vox_cuda_tree *t, const void *samples, const unsigned dim[3], unsigned samplesize,
              const vox_cuda_raw_test *test, cudaStream_t s)
{
    uint64_t V = (uint64_t)dim[0] * dim[1] * dim[2];
    uint64_t bytes = V * samplesize;
    uint64_t mask_bytes = test->mask ? ((1ull << (8 * samplesize)) + 7) / 8 : 0;
    float *P = nullptr;
    uint8_t *d_samples = nullptr, *d_mask = nullptr;
    uint32_t *tile = nullptr, *total = nullptr;
    int rc = VOX_CUDA_OK;
    {
        Dev d(s);
        if (d.get(&d_samples, bytes ? bytes : 1) != cudaSuccess || d.get(&tile, V / SCAN_TILE + 2) != cudaSuccess ||
            d.get(&total, 1) != cudaSuccess || (mask_bytes && d.get(&d_mask, mask_bytes) != cudaSuccess))
            return VOX_CUDA_ENOMEM;
        if (bytes && cudaMemcpyAsync(d_samples, samples, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return VOX_CUDA_ECUDA;
        if (mask_bytes && cudaMemcpyAsync(d_mask, test->mask, mask_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess)
            return VOX_CUDA_ECUDA;
        RawSolid solid{d_samples, d_mask, samplesize, test->lo, test->hi};
        // count the solid voxels first: the set is allocated to size
        uint32_t nt = (uint32_t)((V + SCAN_TILE - 1) / SCAN_TILE);
        uint32_t h_total = 0;
        if (nt) {
            k_tile_sums<<<nt, SCAN_THREADS, 0, s>>>(solid, V, tile);
            count_launch();
            k_scan_tiles<<<1, 1024, 0, s>>>(tile, nt, total);
            count_launch();
            if (cudaMemcpyAsync(&h_total, total, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                cudaStreamSynchronize(s) != cudaSuccess)
                return VOX_CUDA_ECUDA;
        }
        if (h_total) {
            if (cudaMallocAsync(&P, 12ull * h_total, s) != cudaSuccess) return VOX_CUDA_ENOMEM;
            RawPlace place{dim[1], dim[2], vox_voxel[0], vox_voxel[1], vox_voxel[2], P};
            k_tile_apply<<<nt, SCAN_THREADS, 0, s>>>(solid, place, V, tile);
            count_launch();
            if (cudaGetLastError() != cudaSuccess) rc = VOX_CUDA_ECUDA;
        }
        if (rc == VOX_CUDA_OK) rc = build_tree(t, P, h_total, s);
    }
    if (P) cudaFreeAsync(P, s);
    cudaStreamSynchronize(s);
    return rc;
}

int check_raw_args(const unsigned dim[3], unsigned samplesize, const vox_cuda_raw_test *test)
{
    if (!dim || !test || samplesize < 1 || samplesize > 4) return VOX_CUDA_EINVAL;
    if (test->mask && samplesize > 2) return VOX_CUDA_EINVAL;
    uint64_t V = (uint64_t)dim[0] * dim[1] * dim[2];
    if (V > 0xFFFFFFFFull) return VOX_CUDA_ETOOBIG;   // the reference counts samples in an unsigned int
    return VOX_CUDA_OK;
}

}  // namespace

// ======================================================================== API

int build_for_host_tree(const float *set, size_t n, vox_cuda_tree **out, HostTreeExtras *x)
{
    if (n == 0 || n > MAX_VOXELS || !set) return VOX_CUDA_EINVAL;
    return new_tree(out, [&](vox_cuda_tree *t, cudaStream_t s) {
        float *d = nullptr;
        if (cudaMallocAsync(&d, 12ull * n, s) != cudaSuccess) return (int)VOX_CUDA_ENOMEM;
        int rc = VOX_CUDA_OK;
        if (cudaMemcpyAsync(d, set, 12ull * n, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = VOX_CUDA_ECUDA;
        if (rc == VOX_CUDA_OK) rc = build_tree(t, d, n, s, x);
        cudaFreeAsync(d, s);
        cudaStreamSynchronize(s);
        return rc;
    });
}

EXPORT int vox_cuda_tree_build_device(const float *d_set, size_t n, vox_cuda_tree **out)
try {
    if (n && !d_set) return VOX_CUDA_EINVAL;
    return new_tree(out, [&](vox_cuda_tree *t, cudaStream_t s) { return build_tree(t, d_set, n, s); });
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_build(const float *set, size_t n, vox_cuda_tree **out)
try {
    if (n && !set) return VOX_CUDA_EINVAL;
    return new_tree(out, [&](vox_cuda_tree *t, cudaStream_t s) {
        if (n > MAX_VOXELS) return (int)VOX_CUDA_ETOOBIG;
        float *d = nullptr;
        if (n && cudaMallocAsync(&d, 12ull * n, s) != cudaSuccess) return (int)VOX_CUDA_ENOMEM;
        int rc = VOX_CUDA_OK;
        if (n && cudaMemcpyAsync(d, set, 12ull * n, cudaMemcpyHostToDevice, s) != cudaSuccess) rc = VOX_CUDA_ECUDA;
        if (rc == VOX_CUDA_OK) rc = build_tree(t, d, n, s);
        if (d) cudaFreeAsync(d, s);
        cudaStreamSynchronize(s);
        return rc;
    });
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_tree_build_raw(const void *samples, const unsigned dim[3], unsigned samplesize,
                                   const vox_cuda_raw_test *test, vox_cuda_tree **out)
try {
    int rc = check_raw_args(dim, samplesize, test);
    if (rc) return rc;
    if (!samples && (uint64_t)dim[0] * dim[1] * dim[2] != 0) return VOX_CUDA_EINVAL;
    return new_tree(out, [&](vox_cuda_tree *t, cudaStream_t s) {
        return raw_build(t, samples, dim, samplesize, test, s);
    });
} VOX_ABI_FAIL_INT

EXPORT int vox_cuda_read_raw_data(const char *filename, const unsigned dim[3], unsigned samplesize,
                                  const vox_cuda_raw_test *test, vox_cuda_tree **out, const char **error)
try {
    if (out) *out = nullptr;
    int rc = check_raw_args(dim, samplesize, test);
    if (rc || !filename || !out) {
        if (error) *error = "Invalid argument";
        return rc ? rc : VOX_CUDA_EINVAL;
    }
    int fd = open(filename, O_RDONLY);
    if (fd == -1) {
        if (error) *error = strerror(errno);
        return VOX_CUDA_EINVAL;
    }
    struct stat sb;
    if (fstat(fd, &sb) == -1) {
        if (error) *error = strerror(errno);
        close(fd);
        return VOX_CUDA_EINVAL;
    }
    uint64_t bytes = (uint64_t)dim[0] * dim[1] * dim[2] * samplesize;
    if ((uint64_t)sb.st_size != bytes) {   // datareader.c:40-43
        if (error) *error = "Wrong size of dataset";
        close(fd);
        return VOX_CUDA_EINVAL;
    }
    void *buf = nullptr;
    if (bytes && cudaMallocHost(&buf, bytes) != cudaSuccess) {
        close(fd);
        if (error) *error = "Cannot allocate memory";
        return VOX_CUDA_ENOMEM;
    }
    uint64_t got = 0;
    while (got < bytes) {
        ssize_t r = read(fd, static_cast<char *>(buf) + got, (size_t)std::min<uint64_t>(bytes - got, 1u << 30));
        if (r <= 0) {
            if (error) *error = r == 0 ? "Unexpected end of file" : strerror(errno);
            close(fd);
            cudaFreeHost(buf);
            return VOX_CUDA_EINVAL;
        }
        got += (uint64_t)r;
    }
    close(fd);
    rc = vox_cuda_tree_build_raw(buf, dim, samplesize, test, out);
    if (buf) cudaFreeHost(buf);
    if (rc && error) *error = vox_cuda_strerror(rc);
    return rc;
} VOX_ABI_FAIL_INT
