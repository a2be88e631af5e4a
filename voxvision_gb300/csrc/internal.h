/*
 * internal.h -- definitions shared by the translation units of
 * libvoxtrees_cuda (not part of the C ABI).
 */
#ifndef VOX_INTERNAL_H
#define VOX_INTERNAL_H

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <utility>
#include <vector>

#include "flatten.h"
#include "frame_memo.h"
#include "pool_layout.h"
#include "traverse.cuh"
#include "../../include/voxtrees_cuda.h"

using vox::DevTree;

struct vox_cuda_tree {
    int device = 0;
    float bbox[6] = {0, 0, 0, 0, 0, 0};   // root bounding box (for scheduling only)
    uint4 *d_pool = nullptr;
    uint32_t *d_rec_of_id = nullptr;
    uint32_t *d_status = nullptr;          // bit 0: a traversal stack overflowed
    DevTree dev{};
    int cap_class = 0;                     // 0: 28 stack entries, 1: 64, 2: 256
    FlatTree flat;                         // host copy: pre-order table and maps
    size_t pool_bytes = 0;                 // device pool allocation
    size_t map_bytes = 0;                  // device pre-order map allocation
    uint64_t n_nodes = 0, n_units = 0;     // nodes, image units (3 for the empty tree)
    // host node -> pre-order id, sorted by node; built on the first lookup
    std::mutex index_mu;
    bool index_built = false;
    std::vector<std::pair<const vox_node *, uint32_t>> index;
};


// What a device-built image holds (build.cu).
struct ImageStats {
    uint64_t nodes, units, inner, leaf, dense, dots, depth;
    float bbox[6];
    float voxel[3];
};

/* Makes t serve a device image built in place: `pool` (st.units 16-byte
 * units) and `map` (st.nodes pre-order id -> record entries), both
 * cudaMalloc'ed and owned by t from then on; t's previous buffers are freed.
 * st.nodes == 0 (pool and map NULL) is the empty tree.  VOX_CUDA_EDEPTH when
 * the tree is too deep for the traversal stack (the buffers stay the
 * caller's). */
int adopt_image(vox_cuda_tree *t, uint4 *pool, size_t pool_bytes, uint32_t *map, size_t map_bytes,
                const ImageStats &st);

/* What a host tree (struct vox_node) needs beyond the device image when it
 * is rebuilt from a device-built tree: each node's dots_num (an inner or
 * dense node's is in no record) by pre-order id, and the set in the order
 * vox_make_tree leaves it (tree.c sorts its input in place). */
struct HostTreeExtras {
    std::vector<uint32_t> dots_of_id;
    float *order = nullptr;   // 3n floats of host memory, or NULL
};

/* vox_cuda_tree_upload without looking for a device copy vox_make_tree kept
 * (voxtrees_cuda.cu); whether a device tree suits the current device and
 * voxel size. */
int tree_upload_flat(const struct vox_node *root, vox_cuda_tree **out);
bool tree_fits_now(const vox_cuda_tree *t);

/* The tree of the n voxels at `set` (host) built on the GPU into a new
 * handle, with the extras (build.cu). */
int build_for_host_tree(const float *set, size_t n, vox_cuda_tree **out, HostTreeExtras *x);

// Ray stacks hold at most 3 pending children per inner level on the path.
constexpr int CAP0 = 28, CAP1 = 64, CAP2 = 256;

inline int cap_class_for_depth(uint64_t depth)
{
    uint64_t need = 3 * depth + 1;
    if (need <= (uint64_t)CAP0) return 0;
    if (need <= (uint64_t)CAP1) return 1;
    if (need <= (uint64_t)CAP2) return 2;
    return -1;
}

inline cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

inline int status_of(cudaError_t e) { return e == cudaSuccess ? VOX_CUDA_OK : VOX_CUDA_ECUDA; }

/* Adds one to the process-wide kernel launch count (vox_cuda_launch_count). */
void count_launch();

namespace vox {

// k-th index of 0..n-1 taken outward from c: c, c+1, c-1, c+2, ... then the
// rest of the longer side.
__device__ __forceinline__ uint32_t centre_out(uint32_t k, uint32_t c, uint32_t n)
{
    uint32_t m = min(c, n - 1 - c);
    if (k <= 2 * m) return (k & 1) ? c + (k + 1) / 2 : c - k / 2;
    uint32_t j = k - (2 * m + 1);
    return (c < n - 1 - c) ? c + m + 1 + j : c - m - 1 - j;
}

// Work of one BEST frame: the screen rectangle that the tree's bounding box
// can project into (pixels outside it cannot reach the tree and are misses),
// cut in 16x8-pixel block tiles issued outward from the tile where the tree's
// centre projects, and the number of blocks that clear the rest.
struct FramePlan {
    uint32_t x0, y0, x1, y1;     // traced rectangle, multiples of 8 x 4
    uint32_t ntx, nty, ctx, cty; // tiles across / down, tile where the centre projects
    uint32_t ntiles, nclear;     // tracing blocks, clearing blocks
    uint32_t cx0, cy0, cx1, cy1; // where the frame may hold non-zero pixels before the launch: the
                                 // clearing blocks zero this rectangle outside the traced one
};

}  // namespace vox

constexpr int TILE_W = 16, TILE_H = 8;   // render block tile; warps are 8x4

/* The screen rectangle [rect[0], rect[2]) x [rect[1], rect[3]) of a w x h
 * frame outside which no ray can reach the tree (multiples of 8 x 4; empty
 * for an empty tree), and where the tree's centre projects. */
void frame_rect_of(const vox_cuda_tree *t, const vox_cuda_camera &cam, uint32_t w, uint32_t h, uint32_t rect[4],
                   double centre_px[2]);

/* The plan of a BEST frame; cull = false traces the whole frame.
 * Conservative: every pixel whose ray can enter the tree's bounding box lies
 * inside the rectangle. */
void plan_frame(const vox_cuda_tree *t, const vox_cuda_camera &cam, uint32_t w, uint32_t h, bool cull,
                vox::FramePlan &p);
/* The clearing blocks of a plan (plan_frame calls it without a memo). */
void plan_clearing(vox::FramePlan &p, const vox::FrameMemo *memo);


/* The batched frame kernel over a job table the caller allocated for one
 * launch (batch.cu): fills h_table (pinned, frame_job_table_bytes(njobs)
 * bytes, 16-byte aligned), copies it to d_table, zeroes *d_counter and
 * launches, all on s, with `cfg` (tiles 8x4, 1 a grab, 8 blocks per SM --
 * what the autotuner picks for a mix of frames -- when NULL). */
size_t frame_job_table_bytes(uint32_t njobs);
int enqueue_frame_jobs(const vox_cuda_frame_job *jobs, uint32_t njobs, void *h_table, void *d_table,
                       uint32_t *d_counter, int nsm, cudaStream_t s, const vox_cuda_batch_config *cfg = nullptr);

/* The coherent order of a ray batch (raysort.cu): *order (in `scratch`, of
 * ray_order_bytes(n) bytes) lists the rays' indices grouped by direction
 * octant and origin cell; enqueued on s. */
size_t ray_order_bytes(size_t n);
cudaError_t ray_order(const vox_cuda_tree *t, const float *o, const float *d, size_t n, void *scratch,
                      uint32_t **order, cudaStream_t s);
/* The same for a ball batch: grouped by the cell of the centre on a 16^3
 * grid over the tree's box (scratch of ray_order_bytes(n) bytes). */
cudaError_t ball_order(const vox_cuda_tree *t, const float *centres, size_t n, void *scratch, uint32_t **order,
                       cudaStream_t s);

/* Frames one after another in one persistent launch (batch.cu), each
 * announced when complete: flags[j] (host memory the device can write)
 * becomes `epoch` once every store of frame j is visible to the copy engine.
 * d_done: njobs counters the call zeroes on s.  At most 1024 jobs. */
int enqueue_announced_frames(const vox_cuda_frame_job *jobs, uint32_t njobs, void *h_table, void *d_table,
                             uint32_t *d_counter, uint32_t *d_done, uint32_t *flags, uint32_t epoch, int nsm,
                             cudaStream_t s, uint32_t *rects);

#endif
