/*
 * flatten.cpp -- turn a host struct vox_node tree into the device pool image
 * described in pool_layout.h.
 *
 * Two walks: the first numbers the non-NULL nodes in pre-order (node, then
 * children 0..7 -- the numbering the C ABI reports leaves by); the second
 * places records depth first so every subtree is contiguous.  Both walks use
 * explicit work lists, so arbitrarily deep trees do not exhaust the host
 * stack.
 */
#include "flatten.h"

#include <cstring>
#include <vector>

#include "pool_layout.h"

namespace {

inline uint32_t fbits(float f)
{
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

inline bool is_inner(const vox_node *n) { return !(n->flags & VOX_LEAF_MASK); }

struct Placement {
    const vox_node *node;
    uint32_t rec;      // unit offset of the node's record
    uint32_t depth;    // inner nodes above and including this one
};

}  // namespace

int vox_flatten(const vox_node *root, const float voxel[3], FlatTree *out)
{
    out->units.clear();
    out->preorder.clear();
    out->rec_of_id.clear();
    out->index.clear();
    out->n_inner = out->n_leaf = out->n_dense = out->n_dots = out->depth = 0;
    out->voxel[0] = voxel[0];
    out->voxel[1] = voxel[1];
    out->voxel[2] = voxel[2];
    if (!root) return 0;

    // Pass 1: pre-order numbering.
    {
        std::vector<const vox_node *> work{root};
        while (!work.empty()) {
            const vox_node *n = work.back();
            work.pop_back();
            out->index.emplace(n, (uint32_t)out->preorder.size());
            out->preorder.push_back(n);
            if (is_inner(n))
                for (int o = 7; o >= 0; o--)
                    if (n->data.inner.children[o]) work.push_back(n->data.inner.children[o]);
        }
    }
    out->rec_of_id.assign(out->preorder.size(), 0);

    // Pass 2: depth-first placement of 3-unit records.
    std::vector<uint4_host> &u = out->units;
    u.reserve(out->preorder.size() * 4);
    u.resize(VOXP_REC_UNITS);
    std::vector<Placement> work{{root, 0, 0}};
    while (!work.empty()) {
        Placement p = work.back();
        work.pop_back();
        const vox_node *n = p.node;
        uint32_t id = out->index[n];
        out->rec_of_id[id] = p.rec;
        uint32_t meta, link;
        uint4_host extra{0u, 0u, 0u, 0u};
        if (n->flags & VOX_DENSE_LEAF) {
            meta = VOXP_KIND_DENSE;
            link = id;
            out->n_dense++;
        } else if (n->flags & VOX_LEAF) {
            uint32_t cnt = n->dots_num;
            if (cnt >= (1u << 30)) return -1;
            link = (uint32_t)u.size();
            for (uint32_t i = 0; i < cnt; i++)
                u.push_back({fbits(n->data.dots[i][0]), fbits(n->data.dots[i][1]),
                             fbits(n->data.dots[i][2]), 0u});
            meta = VOXP_KIND_LEAF | (cnt << 2);
            extra = {id, cnt, 0u, 0u};
            out->n_leaf++;
            out->n_dots += cnt;
        } else {
            uint32_t mask = 0;
            for (int o = 0; o < 8; o++)
                if (n->data.inner.children[o]) mask |= 1u << o;
            link = (uint32_t)u.size();
            uint32_t nchild = (uint32_t)__builtin_popcount(mask);
            u.resize(u.size() + VOXP_REC_UNITS * nchild);
            uint32_t d = p.depth + 1;
            if (d > out->depth) out->depth = d;
            // Children are placed after this block; push in reverse so octant 0's
            // subtree is laid out first.
            for (int o = 7; o >= 0; o--) {
                const vox_node *ch = n->data.inner.children[o];
                if (!ch) continue;
                uint32_t rank = (uint32_t)__builtin_popcount(mask & ((1u << o) - 1u));
                work.push_back({ch, link + VOXP_REC_UNITS * rank, d});
            }
            meta = VOXP_KIND_INNER | (mask << 8);
            const float *c = n->data.inner.center;
            extra = {fbits(c[0]), fbits(c[1]), fbits(c[2]), 0u};
            out->n_inner++;
        }
        if (u.size() >= VOXP_MAX_UNITS) return -2;
        const vox_box &b = n->bounding_box;
        u[p.rec] = {fbits(b.min[0]), fbits(b.min[1]), fbits(b.min[2]), fbits(b.max[0])};
        u[p.rec + 1] = {fbits(b.max[1]), fbits(b.max[2]), meta, link};
        u[p.rec + 2] = extra;
    }
    return 0;
}

int vox_flatten_validate(const FlatTree &f)
{
    const std::vector<uint4_host> &u = f.units;
    size_t n = u.size();
    if (f.preorder.empty()) return 0;
    if (n < VOXP_REC_UNITS) return -1;
    std::vector<uint32_t> work{0};
    size_t seen = 0;
    while (!work.empty()) {
        uint32_t rec = work.back();
        work.pop_back();
        if ((size_t)rec + VOXP_REC_UNITS > n) return -1;
        seen++;
        uint32_t meta = u[rec + 1].z, link = u[rec + 1].w;
        uint32_t kind = meta & 3u;
        if (kind == VOXP_KIND_DENSE) {
            if (link >= f.preorder.size()) return -1;
        } else if (kind == VOXP_KIND_LEAF) {
            uint64_t cnt = meta >> 2;
            if ((uint64_t)link + cnt > n) return -1;
            if (u[rec + 2].x >= f.preorder.size() || u[rec + 2].y != cnt) return -1;
        } else if (kind == VOXP_KIND_INNER) {
            uint32_t mask = (meta >> 8) & 0xFFu;
            uint32_t k = (uint32_t)__builtin_popcount(mask);
            if ((uint64_t)link + (uint64_t)VOXP_REC_UNITS * k > n) return -1;
            for (uint32_t i = 0; i < k; i++) work.push_back(link + VOXP_REC_UNITS * i);
        } else {
            return -1;
        }
        if (seen > f.preorder.size()) return -1;
    }
    return seen == f.preorder.size() ? 0 : -1;
}
