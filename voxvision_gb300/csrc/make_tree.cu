/*
 * make_tree.cu -- vox_make_tree (tree.h:60, tree.c:249-338) with the
 * reference's signature and result, for large sets built on the GPU.
 *
 * A set of at least vox_cuda_make_tree_gpu_min voxels (65,536 unless set) is
 * built on the GPU (build.cu), which gives the device image of the tree, each
 * node's dots_num and the set in the order tree.c leaves it (it sorts its
 * input in place).  The host tree is then made from the image on all host
 * threads: every node allocated as the host build allocates it (leaves with
 * room for VOX_MAX_DOTS voxels, overflowed leaves for all of theirs), the
 * same flags, boxes, centres, children and voxels -- node for node the tree
 * vox_make_tree_host builds.  The device copy is kept for the tree's first
 * vox_cuda_tree_upload (or single query, or render context), which then
 * costs nothing; an edit or vox_destroy_tree drops it.  Without a usable GPU,
 * or if any step fails, the host build runs.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "internal.h"
#include "abi_guard.h"
#include "parallel.h"

#define EXPORT extern "C" __attribute__((visibility("default")))

extern "C" struct vox_node *vox_make_tree_host(vox_dot set[], size_t n);
void dropin_keep_prebuilt(const vox_node *root, vox_cuda_tree *t) noexcept;

namespace {

std::atomic<size_t> g_gpu_min{65536};

bool have_gpu()
{
    static std::once_flag once;
    static int count = 0;
    std::call_once(once, [] {
        if (cudaGetDeviceCount(&count) != cudaSuccess) {
            count = 0;
            cudaGetLastError();
        }
    });
    return count > 0;
}

inline float fl(uint32_t u)
{
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

void free_nodes(std::vector<vox_node *> &nd)
{
    for (vox_node *p : nd) {
        if (!p) continue;
        if ((p->flags & VOX_LEAF) && !(p->flags & VOX_DENSE_LEAF)) std::free(p->data.dots);
        std::free(p);
    }
}

// The host tree of a device image (pool_layout.h): nu units, pre-order id
// -> record offset for `nodes` nodes, and dots_num by pre-order id.  Node
// pointers in pre-order go to `pre`.  NULL when an allocation fails.
vox_node *tree_from_image(const uint4_host *u, size_t nu, const uint32_t *rec_of_id, size_t nodes,
                          const std::vector<uint32_t> &dots, std::vector<const vox_node *> &pre)
{
    constexpr size_t CHUNK = 4096;
    const size_t nchunk = (nodes + CHUNK - 1) / CHUNK;
    pre.reserve(nodes);   // every allocation that may throw comes before the nodes'
    // record offset -> pre-order id, written (and read) at node records only
    std::unique_ptr<uint32_t[]> id_of_rec(new uint32_t[nu]);
    parallel_for(nchunk, [&](size_t c) {
        for (size_t id = c * CHUNK; id < std::min(nodes, (c + 1) * CHUNK); id++)
            id_of_rec[rec_of_id[id]] = (uint32_t)id;
    });
    std::vector<vox_node *> nd(nodes, nullptr);
    std::atomic<bool> ok{true};
    parallel_for(nchunk, [&](size_t c) {
        for (size_t id = c * CHUNK; id < std::min(nodes, (c + 1) * CHUNK) && ok.load(); id++) {
            const uint32_t r = rec_of_id[id];
            const uint4_host &r0 = u[r], &r1 = u[r + 1], &r2 = u[r + 2];
            vox_node *p = static_cast<vox_node *>(std::calloc(1, sizeof(vox_node)));
            if (!p) {
                ok = false;
                return;
            }
            nd[id] = p;
            p->bounding_box.min[0] = fl(r0.x);
            p->bounding_box.min[1] = fl(r0.y);
            p->bounding_box.min[2] = fl(r0.z);
            p->bounding_box.max[0] = fl(r0.w);
            p->bounding_box.max[1] = fl(r1.x);
            p->bounding_box.max[2] = fl(r1.y);
            const uint32_t meta = r1.z, link = r1.w, kind = meta & 3u;
            if (kind == VOXP_KIND_DENSE) {
                p->flags = VOX_DENSE_LEAF;
                p->dots_num = dots[id];
            } else if (kind == VOXP_KIND_LEAF) {
                uint32_t cnt = meta >> 2;
                p->flags = VOX_LEAF | (cnt > VOX_MAX_DOTS ? VOX_OVERFLOW : 0u);   // tree.c:281-305
                p->dots_num = cnt;
                size_t cap = cnt > VOX_MAX_DOTS ? cnt : VOX_MAX_DOTS;
                p->data.dots = static_cast<vox_dot *>(std::malloc(cap * sizeof(vox_dot)));
                if (!p->data.dots) {
                    p->flags = 0;   // nothing to free for it
                    ok = false;
                    return;
                }
                for (uint32_t i = 0; i < cnt; i++) {
                    const uint4_host &v = u[link + i];
                    p->data.dots[i][0] = fl(v.x);
                    p->data.dots[i][1] = fl(v.y);
                    p->data.dots[i][2] = fl(v.z);
                }
            } else {
                p->flags = 0;
                p->dots_num = dots[id];
                p->data.inner.center[0] = fl(r2.x);
                p->data.inner.center[1] = fl(r2.y);
                p->data.inner.center[2] = fl(r2.z);
            }
        }
    });
    if (!ok) {
        free_nodes(nd);
        return nullptr;
    }
    parallel_for(nchunk, [&](size_t c) {   // children: the records of an inner node's child block
        for (size_t id = c * CHUNK; id < std::min(nodes, (c + 1) * CHUNK); id++) {
            const uint4_host &r1 = u[rec_of_id[id] + 1];
            if ((r1.z & 3u) != VOXP_KIND_INNER) continue;
            uint32_t mask = (r1.z >> 8) & 0xFFu, link = r1.w, j = 0;
            for (int o = 0; o < 8; o++)
                if (mask & (1u << o)) nd[id]->data.inner.children[o] = nd[id_of_rec[link + VOXP_REC_UNITS * j++]];
        }
    });
    pre.assign(nd.begin(), nd.end());
    return nd[0];
}

// NULL (and nothing left allocated) if any step fails or throws.  The large
// buffers (the set's final order, the image) are left uninitialised until
// the copies fill them, and the final order goes back into `set` on all host
// threads: on the 13.9 M-voxel set this cut the call from 131-140 ms to
// 104-107 ms (the GPU build and the copies about 47, the host nodes, each
// allocated on its own as the host build allocates it, most of the rest).
vox_node *make_on_gpu(vox_dot set[], size_t n)
{
    std::unique_ptr<float[]> order(new float[3 * n]);
    HostTreeExtras x;
    x.order = order.get();
    struct Owned {
        vox_cuda_tree *t = nullptr;
        ~Owned() { if (t) vox_cuda_tree_free(t); }
    } own;
    if (build_for_host_tree(&set[0][0], n, &own.t, &x) != VOX_CUDA_OK) return nullptr;
    size_t nu = 0, ni = 0;
    vox_cuda_tree_image(own.t, nullptr, 0, nullptr, 0, &nu, &ni);
    std::unique_ptr<uint4_host[]> units(new uint4_host[nu ? nu : 1]);
    std::unique_ptr<uint32_t[]> recs(new uint32_t[ni ? ni : 1]);
    std::vector<const vox_node *> pre;
    vox_node *root = nullptr;
    if (ni && ni == x.dots_of_id.size() &&
        vox_cuda_tree_image(own.t, units.get(), nu, recs.get(), ni, nullptr, nullptr) == VOX_CUDA_OK)
        root = tree_from_image(units.get(), nu, recs.get(), ni, x.dots_of_id, pre);
    if (!root) return nullptr;
    // nothing below throws
    vox_cuda_tree *t = own.t;
    own.t = nullptr;
    t->flat.preorder = std::move(pre);
    dropin_keep_prebuilt(root, t);
    constexpr size_t PART = size_t(1) << 20;   // voxels a host thread copies at a time
    parallel_for((n + PART - 1) / PART, [&](size_t c) {
        const size_t a = c * PART, b = std::min(n, a + PART);
        std::memcpy(&set[a][0], order.get() + 3 * a, 12 * (b - a));
    });
    return root;
}

}  // namespace

EXPORT size_t vox_cuda_make_tree_gpu_min(size_t n) { return g_gpu_min.exchange(n); }

EXPORT struct vox_node *vox_make_tree(vox_dot set[], size_t n)
try {
    if (n == 0) return nullptr;
    if (set && n >= g_gpu_min.load() && n <= 0x7FFFFFFFull && have_gpu()) {
        vox_node *root = nullptr;
        try {
            root = make_on_gpu(set, n);
        } catch (...) {
            root = nullptr;   // host memory ran short: the host build may still fit
        }
        if (root) return root;
    }
    return vox_make_tree_host(set, n);
} VOX_ABI_FAIL_NULL
