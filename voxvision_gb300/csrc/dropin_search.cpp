/*
 * dropin_search.cpp -- vox_ray_tree_intersection and vox_tree_ball_collidep
 * with the reference's signatures (src/voxtrees/search.h:24-26, :36-37),
 * answered on the GPU.
 *
 * The reference accepts any node as the search root (renderer.c:297 passes a
 * leaf).  A registry of uploaded trees maps a node pointer to (device tree,
 * pre-order id); a pointer found in no registered tree is taken as the root
 * of a new tree and uploaded.  The library's vox_insert_voxel and
 * vox_delete_voxel drop the copies of the trees they edit; trees edited by
 * other code must be dropped with vox_cuda_forget_tree before the next
 * search.  These single-query calls
 * cost a round trip each; batches belong in vox_cuda_ray_batch.
 */
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/voxtrees.h"
#include "../../include/voxtrees_cuda.h"
#include "abi_guard.h"

#define EXPORT extern "C" __attribute__((visibility("default")))

// voxtrees_cuda.cu: the upload proper (flatten and copy), and whether a device
// tree matches the current device and voxel size.
int tree_upload_flat(const vox_node *root, vox_cuda_tree **out);
bool tree_fits_now(const vox_cuda_tree *t);

namespace {

struct Entry {
    const vox_node *root;
    vox_cuda_tree *tree;
};

std::mutex g_mu;
std::vector<Entry> g_trees;
// Device copies made by vox_make_tree when it built the tree on the GPU,
// waiting for the first vox_cuda_tree_upload (or single query) of the root.
std::vector<Entry> g_prebuilt;

vox_cuda_tree *take_prebuilt_locked(const vox_node *root)
{
    for (size_t i = 0; i < g_prebuilt.size(); i++) {
        if (g_prebuilt[i].root == root) {
            vox_cuda_tree *t = g_prebuilt[i].tree;
            g_prebuilt[i] = g_prebuilt.back();
            g_prebuilt.pop_back();
            return t;
        }
    }
    return nullptr;
}

// The device copy vox_make_tree made of the tree at `root`, for its first
// upload; a copy made for another device or another voxel size is dropped.
vox_cuda_tree *take_prebuilt_usable_locked(const vox_node *root)
{
    vox_cuda_tree *t = take_prebuilt_locked(root);
    if (!t || tree_fits_now(t)) return t;
    vox_cuda_tree_free(t);
    return nullptr;
}

// Device tree holding `node` and the node's pre-order id, uploading a new
// tree rooted at `node` when no registered tree contains it.
bool resolve(const vox_node *node, vox_cuda_tree **tree, uint32_t *id)
{
    std::lock_guard<std::mutex> lock(g_mu);
    for (const Entry &e : g_trees) {
        if (vox_cuda_tree_node_id(e.tree, node, id) == VOX_CUDA_OK) {
            *tree = e.tree;
            return true;
        }
    }
    vox_cuda_tree *t = take_prebuilt_usable_locked(node);
    if (!t && tree_upload_flat(node, &t) != VOX_CUDA_OK) return false;
    try {
        g_trees.push_back({node, t});
    } catch (...) {
        vox_cuda_tree_free(t);
        throw;
    }
    *tree = t;
    *id = 0;
    return true;
}

}  // namespace

EXPORT const struct vox_node *vox_ray_tree_intersection(const struct vox_node *tree, const vox_dot origin,
                                                        const vox_dot dir, vox_dot res)
try {
    if (!tree) return nullptr;
    vox_cuda_tree *t;
    uint32_t id;
    if (!resolve(tree, &t, &id)) return nullptr;
    uint32_t leaf = VOX_CUDA_MISS;
    if (vox_cuda_ray_batch(t, origin, dir, id ? &id : nullptr, 1, &leaf, nullptr, res, nullptr) != VOX_CUDA_OK)
        return nullptr;
    return leaf == VOX_CUDA_MISS ? nullptr : vox_cuda_tree_node(t, leaf);
} VOX_ABI_FAIL_NULL

EXPORT int vox_tree_ball_collidep(const struct vox_node *tree, const vox_dot center, float radius)
try {
    if (!tree) return 0;
    vox_cuda_tree *t;
    uint32_t id;
    if (!resolve(tree, &t, &id)) return 0;
    if (id != 0) {
        // A ball query below the root: upload that subtree on its own.
        std::lock_guard<std::mutex> lock(g_mu);
        vox_cuda_tree *sub = nullptr;
        if (vox_cuda_tree_upload(tree, &sub) != VOX_CUDA_OK) return 0;
        uint8_t hit = 0;
        int rc = vox_cuda_ball_batch(sub, center, &radius, 1, &hit, nullptr);
        vox_cuda_tree_free(sub);
        return rc == VOX_CUDA_OK ? hit : 0;
    }
    uint8_t hit = 0;
    if (vox_cuda_ball_batch(t, center, &radius, 1, &hit, nullptr) != VOX_CUDA_OK) return 0;
    return hit;
} VOX_ABI_FAIL_ZERO

EXPORT void vox_cuda_forget_tree(const struct vox_node *root)
try {
    std::lock_guard<std::mutex> lock(g_mu);
    if (vox_cuda_tree *p = take_prebuilt_locked(root)) vox_cuda_tree_free(p);
    for (size_t i = 0; i < g_trees.size(); i++) {
        if (g_trees[i].root == root) {
            vox_cuda_tree_free(g_trees[i].tree);
            g_trees.erase(g_trees.begin() + (long)i);
            return;
        }
    }
} VOX_ABI_FAIL_VOID

// Every cached device copy dropped (g_mu held).
static void forget_all_locked()
{
    for (Entry &e : g_prebuilt) vox_cuda_tree_free(e.tree);
    for (Entry &e : g_trees) vox_cuda_tree_free(e.tree);
    g_prebuilt.clear();
    g_trees.clear();
}

// The cached device copies of trees that contain `node` dropped (g_mu held).
static void forget_containing_locked(const struct vox_node *node)
{
    for (size_t i = 0; i < g_prebuilt.size();) {
        uint32_t id;
        if (vox_cuda_tree_node_id(g_prebuilt[i].tree, node, &id) == VOX_CUDA_OK) {
            vox_cuda_tree_free(g_prebuilt[i].tree);
            g_prebuilt[i] = g_prebuilt.back();
            g_prebuilt.pop_back();
        } else {
            i++;
        }
    }
    for (size_t i = 0; i < g_trees.size();) {
        uint32_t id;
        if (vox_cuda_tree_node_id(g_trees[i].tree, node, &id) == VOX_CUDA_OK) {
            vox_cuda_tree_free(g_trees[i].tree);
            g_trees[i] = g_trees.back();
            g_trees.pop_back();
        } else {
            i++;
        }
    }
}

// Called by the tree-editing functions before they change a tree: a cached
// device copy of any tree that contains `node` is dropped.  If the node
// lookup cannot be made (its index could not be allocated), every copy is
// dropped: a later query uploads again.
extern "C" void vox_dropin_forget_containing(const struct vox_node *node)
{
    std::lock_guard<std::mutex> lock(g_mu);
    try {
        forget_containing_locked(node);
    } catch (...) {
        forget_all_locked();
    }
}

// vox_make_tree (make_tree.cu): keep the device copy of a tree it built on
// the GPU until the tree's first upload, edit or destruction (or free it, if
// it cannot be kept: it only saves that upload).
void dropin_keep_prebuilt(const vox_node *root, vox_cuda_tree *t) noexcept
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (vox_cuda_tree *old = take_prebuilt_locked(root)) vox_cuda_tree_free(old);
    try {
        g_prebuilt.push_back({root, t});
    } catch (...) {
        vox_cuda_tree_free(t);
    }
}

// vox_cuda_tree_upload: the kept device copy of `root`, if there is one.
vox_cuda_tree *dropin_take_prebuilt(const vox_node *root)
{
    std::lock_guard<std::mutex> lock(g_mu);
    return take_prebuilt_usable_locked(root);
}
