/*
 * flatten.cpp -- turn a host struct vox_node tree into the device pool image
 * described in pool_layout.h.  Trees of either vox_dot layout are read: the
 * scalar one (float[3]) and the SSE one (float[4] aligned to 16, vox_node16);
 * the image is the same for the same nodes.
 *
 * Layout.  Records are placed depth first: when a node is visited (in
 * pre-order: node, then children 0..7), its child block -- or its voxel run,
 * for a leaf -- is appended to the image.  So the image region a subtree
 * appends is contiguous, starts where the subtree's root is visited and has
 * a size known in advance: 3 units per node below the subtree's root plus its
 * leaves' voxels; and its nodes' pre-order ids are consecutive.  The
 * pre-order numbering is the one the C ABI reports leaves by.
 *
 * Parallel walk.  The host tree is pointer-chased node by node (every node
 * its own allocation), which makes one thread slow on large trees.  The walk
 * therefore cuts the tree a few levels down: the nodes above the cut are
 * visited by one thread, which reserves for every subtree below the cut its
 * id range and image region from a counting pass; the subtrees are then
 * counted, placed and validated by all host threads, each writing only its
 * own ranges.  The image is the same as a single depth-first walk's.  Work
 * lists are explicit, so arbitrarily deep trees do not exhaust the stack.
 */
#include "flatten.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "pool_layout.h"
#include "parallel.h"

namespace {

inline uint32_t fbits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

struct Sizes {
    uint64_t nodes = 0, units = 0, inner = 0, leaf = 0, dense = 0, dots = 0, depth = 0;
};

// Every walk below is a template over the node layout N (vox_node: scalar
// vox_dot; vox_node16: the SSE layout); both have the same member names.

// Nodes of the subtree, units it appends (child blocks and voxel runs), kinds,
// and its depth in inner nodes.
template <class N>
Sizes count(const N *root)
{
    Sizes s;
    std::vector<std::pair<const N *, uint32_t>> work{{root, 0}};
    while (!work.empty()) {
        auto [n, d] = work.back();
        work.pop_back();
        s.nodes++;
        if (n->flags & VOX_DENSE_LEAF) {
            s.dense++;
        } else if (n->flags & VOX_LEAF) {
            s.leaf++;
            s.dots += n->dots_num;
            s.units += n->dots_num;
        } else {
            s.inner++;
            s.depth = std::max<uint64_t>(s.depth, d + 1);
            for (int o = 0; o < 8; o++)
                if (const N *ch = n->data.inner.children[o]) {
                    s.units += VOXP_REC_UNITS;
                    work.push_back({ch, d + 1});
                }
        }
    }
    return s;
}

// A subtree placed on its own: its root's record offset (in its parent's
// child block), its first pre-order id and the start of its image region.
template <class N>
struct Task {
    const N *node;
    uint32_t rec, id, next;
};

// Writes the record of node n at `rec` (id `id`); for an inner node or a
// leaf, appends its child block or voxel run at *next.  Pushes the children
// (in reverse octant order, so they are visited in pre-order) onto `work`.
// Returns false if a leaf is too large for the record format.
template <class N>
bool place(const N *n, uint32_t rec, uint32_t id, uint32_t *next, uint4_host *u,
           std::vector<std::pair<const N *, uint32_t>> *work)
{
    uint32_t meta, link;
    uint4_host extra{0u, 0u, 0u, 0u};
    if (n->flags & VOX_DENSE_LEAF) {
        meta = VOXP_KIND_DENSE;
        link = id;
    } else if (n->flags & VOX_LEAF) {
        uint32_t cnt = n->dots_num;
        if (cnt >= (1u << 30)) return false;
        link = *next;
        for (uint32_t i = 0; i < cnt; i++)
            u[(*next)++] = {fbits(n->data.dots[i][0]), fbits(n->data.dots[i][1]), fbits(n->data.dots[i][2]), 0u};
        meta = VOXP_KIND_LEAF | (cnt << 2);
        extra = {id, cnt, 0u, 0u};
    } else {
        uint32_t mask = 0;
        for (int o = 0; o < 8; o++)
            if (n->data.inner.children[o]) mask |= 1u << o;
        link = *next;
        *next += VOXP_REC_UNITS * (uint32_t)__builtin_popcount(mask);
        for (int o = 7; o >= 0; o--) {
            const N *ch = n->data.inner.children[o];
            if (!ch) continue;
            uint32_t rank = (uint32_t)__builtin_popcount(mask & ((1u << o) - 1u));
            work->push_back({ch, link + VOXP_REC_UNITS * rank});
        }
        meta = VOXP_KIND_INNER | (mask << 8);
        const float *c = n->data.inner.center;
        extra = {fbits(c[0]), fbits(c[1]), fbits(c[2]), 0u};
    }
    const auto &b = n->bounding_box;
    u[rec] = {fbits(b.min[0]), fbits(b.min[1]), fbits(b.min[2]), fbits(b.max[0])};
    u[rec + 1] = {fbits(b.max[1]), fbits(b.max[2]), meta, link};
    u[rec + 2] = extra;
    return true;
}

// Places a whole subtree depth first from its task.
template <class N>
bool place_subtree(const Task<N> &t, FlatTree *out)
{
    std::vector<std::pair<const N *, uint32_t>> work{{t.node, t.rec}};
    uint32_t id = t.id, next = t.next;
    uint4_host *u = out->units.data();
    while (!work.empty()) {
        auto [n, rec] = work.back();
        work.pop_back();
        out->preorder[id] = reinterpret_cast<const vox_node *>(n);
        out->rec_of_id[id] = rec;
        if (!place(n, rec, id, &next, u, &work)) return false;
        id++;
    }
    return true;
}

constexpr uint32_t CUT_DEPTH = 3;   // levels walked by one thread (up to 512 subtrees below)

template <class N>
int flatten_tree(const N *root, const float voxel[3], FlatTree *out)
{
    out->units.clear();
    out->preorder.clear();
    out->rec_of_id.clear();
    out->n_inner = out->n_leaf = out->n_dense = out->n_dots = out->depth = 0;
    out->voxel[0] = voxel[0];
    out->voxel[1] = voxel[1];
    out->voxel[2] = voxel[2];
    if (!root) return 0;

    // 1. The subtrees at the cut depth, in pre-order, counted in parallel;
    //    the nodes above the cut counted here.
    std::vector<const N *> cut;
    Sizes top;
    {
        std::vector<std::pair<const N *, uint32_t>> work{{root, 0}};
        while (!work.empty()) {
            auto [n, d] = work.back();
            work.pop_back();
            if (d == CUT_DEPTH) { cut.push_back(n); continue; }
            top.nodes++;
            if (n->flags & VOX_DENSE_LEAF) {
                top.dense++;
            } else if (n->flags & VOX_LEAF) {
                top.leaf++;
                top.dots += n->dots_num;
                top.units += n->dots_num;
            } else {
                top.inner++;
                top.depth = std::max<uint64_t>(top.depth, d + 1);
                for (int o = 7; o >= 0; o--)
                    if (const N *ch = n->data.inner.children[o]) {
                        top.units += VOXP_REC_UNITS;
                        work.push_back({ch, d + 1});
                    }
            }
        }
    }
    std::vector<Sizes> sizes(cut.size());
    parallel_for(cut.size(), [&](size_t i) { sizes[i] = count(cut[i]); });
    uint64_t n_nodes = top.nodes, n_units = VOXP_REC_UNITS + top.units;
    out->n_inner = top.inner; out->n_leaf = top.leaf; out->n_dense = top.dense; out->n_dots = top.dots;
    out->depth = top.depth;
    for (const Sizes &z : sizes) {
        n_nodes += z.nodes;
        n_units += z.units;
        out->n_inner += z.inner; out->n_leaf += z.leaf; out->n_dense += z.dense; out->n_dots += z.dots;
        if (z.depth) out->depth = std::max<uint64_t>(out->depth, CUT_DEPTH + z.depth);
    }
    if (n_units >= VOXP_MAX_UNITS || n_nodes >= 0xFFFFFFFFull) return -2;
    out->preorder.resize(n_nodes);
    out->rec_of_id.resize(n_nodes);
    out->units.resize(n_units);

    // 2. The levels above the cut, depth first, reserving each cut subtree's
    //    id range and image region where the single walk would place it.
    std::vector<Task<N>> tasks;
    tasks.reserve(cut.size());
    {
        std::vector<std::pair<const N *, uint32_t>> work{{root, 0}}, kids;
        std::vector<uint32_t> depth{0};
        uint32_t id = 0, next = VOXP_REC_UNITS;
        size_t k = 0;
        uint4_host *u = out->units.data();
        while (!work.empty()) {
            auto [n, rec] = work.back();
            work.pop_back();
            uint32_t d = depth.back();
            depth.pop_back();
            if (d == CUT_DEPTH) {
                const Sizes &z = sizes[k++];
                tasks.push_back({n, rec, id, next});
                id += (uint32_t)z.nodes;
                next += (uint32_t)z.units;
                continue;
            }
            out->preorder[id] = reinterpret_cast<const vox_node *>(n);
            out->rec_of_id[id] = rec;
            kids.clear();
            if (!place(n, rec, id, &next, u, &kids)) return -1;
            for (auto &c : kids) {
                work.push_back(c);
                depth.push_back(d + 1);
            }
            id++;
        }
    }

    // 3. The subtrees, in parallel.
    std::atomic<bool> ok{true};
    parallel_for(tasks.size(), [&](size_t i) {
        if (!place_subtree(tasks[i], out)) ok = false;
    });
    return ok ? 0 : -1;
}

}  // namespace

int vox_flatten(const vox_node *root, const float voxel[3], FlatTree *out)
{
    return flatten_tree(root, voxel, out);
}

int vox_flatten16(const vox_node16 *root, const float voxel[3], FlatTree *out)
{
    return flatten_tree(root, voxel, out);
}

namespace {

// Walks the image below record `rec`, checking offsets and kinds; counts
// the records reached.  False as soon as something is out of place or more
// records are reached than the tree has.
bool check_subtree(const FlatTree &f, uint32_t rec, uint64_t *seen)
{
    const std::vector<uint4_host> &u = f.units;
    size_t n = u.size();
    std::vector<uint32_t> work{rec};
    while (!work.empty()) {
        uint32_t r = work.back();
        work.pop_back();
        if ((size_t)r + VOXP_REC_UNITS > n) return false;
        if (++*seen > f.preorder.size()) return false;
        uint32_t meta = u[r + 1].z, link = u[r + 1].w;
        uint32_t kind = meta & 3u;
        if (kind == VOXP_KIND_DENSE) {
            if (link >= f.preorder.size()) return false;
        } else if (kind == VOXP_KIND_LEAF) {
            uint64_t cnt = meta >> 2;
            if ((uint64_t)link + cnt > n) return false;
            if (u[r + 2].x >= f.preorder.size() || u[r + 2].y != cnt) return false;
        } else if (kind == VOXP_KIND_INNER) {
            uint32_t mask = (meta >> 8) & 0xFFu;
            uint32_t k = (uint32_t)__builtin_popcount(mask);
            if ((uint64_t)link + (uint64_t)VOXP_REC_UNITS * k > n) return false;
            for (uint32_t i = 0; i < k; i++) work.push_back(link + VOXP_REC_UNITS * i);
        } else {
            return false;
        }
    }
    return true;
}

}  // namespace

int vox_flatten_validate(const FlatTree &f)
{
    if (f.preorder.empty()) return 0;
    const std::vector<uint4_host> &u = f.units;
    if (u.size() < VOXP_REC_UNITS) return -1;
    // the records a few levels down, checked level by level here ...
    std::vector<uint32_t> level{0};
    uint64_t seen = 0;
    for (uint32_t d = 0; d < CUT_DEPTH && !level.empty(); d++) {
        std::vector<uint32_t> below;
        for (uint32_t r : level) {
            if ((size_t)r + VOXP_REC_UNITS > u.size()) return -1;
            seen++;
            uint32_t meta = u[r + 1].z, link = u[r + 1].w;
            uint32_t kind = meta & 3u;
            if (kind == VOXP_KIND_INNER) {
                uint32_t k = (uint32_t)__builtin_popcount((meta >> 8) & 0xFFu);
                if ((uint64_t)link + (uint64_t)VOXP_REC_UNITS * k > u.size()) return -1;
                for (uint32_t i = 0; i < k; i++) below.push_back(link + VOXP_REC_UNITS * i);
            } else {
                uint64_t before = seen - 1, s = 0;
                if (!check_subtree(f, r, &s)) return -1;   // a leaf: checked whole
                seen = before + s;
            }
        }
        level.swap(below);
    }
    if (seen > f.preorder.size()) return -1;
    // ... and the subtrees below them in parallel
    std::vector<uint64_t> counts(level.size(), 0);
    std::atomic<bool> ok{true};
    parallel_for(level.size(), [&](size_t i) {
        if (!check_subtree(f, level[i], &counts[i])) ok = false;
    });
    if (!ok) return -1;
    for (uint64_t c : counts) seen += c;
    return seen == f.preorder.size() ? 0 : -1;
}
