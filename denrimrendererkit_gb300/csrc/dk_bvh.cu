// Traversal BVH of the sm_103a path tracer (host side).
//
// The reference traverses its median-split binary BVH (BVHBuilder.swift:7-135)
// left child first with a strict `t < closest.t` (PathTrace.metal:3340-3395),
// so among hits at equal distance it returns the triangle that comes first in
// left-first DFS leaf order.  That order is the only thing this backend takes
// from the caller's BVH: `referenceSlots` numbers every triangle reachable from
// the caller's tree by its DFS leaf position.  Traversal itself runs over a
// binned-SAH binary tree built here (`buildSahTraversal`); the kernels return
// the argmin over (t, slot), which is the reference's answer.
//
// Output layout (see dk_kernels.h): the binary SAH tree collapsed into 4-wide
// nodes of 8 x float4 (the x, y, z slabs of four children, one lane each, and
// the four child references: interior index, or 0x80000000 | first << 3 |
// (count - 1) for a leaf of <= 8 slots); 3 x float4 per leaf slot: (v0,
// reference slot), (v1 - v0, triangle index), (v2 - v0, flags: bit 0 = blocks
// shadow rays, bits 8..15 material ID); one dummy slot at the end.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <future>
#include <memory>
#include <string>
#include <vector>

#include "dk_kernels.h"

namespace dk {

namespace {

constexpr uint32_t kLeaf = 0x80000000u;
constexpr uint32_t kMaxLeaf = 8;
constexpr int kBins = 32;

inline float asFloat(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

struct Prim {
    float mn[3], mx[3], c[3];
    uint32_t tri;
};

struct Box {
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const float* lo, const float* hi) {
        for (int a = 0; a < 3; ++a) {
            mn[a] = std::fmin(mn[a], lo[a]);
            mx[a] = std::fmax(mx[a], hi[a]);
        }
    }
    void grow(const Box& b) { grow(b.mn, b.mx); }
    float halfArea() const {
        if (mn[0] > mx[0]) return 0.0f;
        float dx = mx[0] - mn[0], dy = mx[1] - mn[1], dz = mx[2] - mn[2];
        return dx * dy + dy * dz + dz * dx;
    }
};

struct TNode {
    Box box;
    std::unique_ptr<TNode> l, r;
    uint32_t first = 0, count = 0;
};

std::unique_ptr<TNode> build(Prim* p, uint32_t first, uint32_t n, int depth) {
    auto node = std::make_unique<TNode>();
    Box cb;
    for (uint32_t i = first; i < first + n; ++i) {
        node->box.grow(p[i].mn, p[i].mx);
        cb.grow(p[i].c, p[i].c);
    }
    auto makeLeaf = [&]() {
        node->first = first;
        node->count = n;
        return std::move(node);
    };
    if (n == 1) return makeLeaf();
    // Binned SAH over the three axes (traversal cost 1, intersection cost 1).
    float bestCost = FLT_MAX;
    int bestAxis = -1, bestSplit = -1;
    for (int a = 0; a < 3; ++a) {
        float ext = cb.mx[a] - cb.mn[a];
        if (!(ext > 0.0f)) continue;
        Box bins[kBins];
        uint32_t counts[kBins] = {};
        float scale = (float)kBins / ext;
        for (uint32_t i = first; i < first + n; ++i) {
            int b = std::min(kBins - 1, (int)((p[i].c[a] - cb.mn[a]) * scale));
            bins[b].grow(p[i].mn, p[i].mx);
            ++counts[b];
        }
        float rightArea[kBins];
        uint32_t rightCount[kBins];
        Box acc;
        uint32_t cnt = 0;
        for (int b = kBins - 1; b > 0; --b) {
            acc.grow(bins[b]);
            cnt += counts[b];
            rightArea[b] = acc.halfArea();
            rightCount[b] = cnt;
        }
        acc = Box();
        cnt = 0;
        for (int b = 0; b < kBins - 1; ++b) {
            acc.grow(bins[b]);
            cnt += counts[b];
            if (cnt == 0 || rightCount[b + 1] == 0) continue;
            float cost = acc.halfArea() * (float)cnt + rightArea[b + 1] * (float)rightCount[b + 1];
            if (cost < bestCost) {
                bestCost = cost;
                bestAxis = a;
                bestSplit = b;
            }
        }
    }
    float nodeArea = node->box.halfArea();
    float splitCost = 1.0f + (nodeArea > 0.0f ? bestCost / nodeArea : 0.0f);
    if (n <= kMaxLeaf && (bestAxis < 0 || (float)n <= splitCost)) return makeLeaf();
    uint32_t mid;
    if (bestAxis < 0) {  // coincident centroids: split the range in half
        mid = first + n / 2;
    } else {
        float ext = cb.mx[bestAxis] - cb.mn[bestAxis];
        float scale = (float)kBins / ext;
        float lo = cb.mn[bestAxis];
        int a = bestAxis, s = bestSplit;
        Prim* m = std::partition(p + first, p + first + n, [=](const Prim& q) {
            return std::min(kBins - 1, (int)((q.c[a] - lo) * scale)) <= s;
        });
        mid = (uint32_t)(m - p);
        if (mid == first || mid == first + n) mid = first + n / 2;
    }
    if (n > 65536 && depth < 6) {
        auto fut = std::async(std::launch::async, [=] { return build(p, first, mid - first, depth + 1); });
        node->r = build(p, mid, first + n - mid, depth + 1);
        node->l = fut.get();
    } else {
        node->l = build(p, first, mid - first, depth + 1);
        node->r = build(p, mid, first + n - mid, depth + 1);
    }
    return node;
}

// 4-wide node record (8 x float4): child boxes as x-min, x-max, y-min, y-max,
// z-min, z-max rows (one lane per child), the four child references, a spare
// row.  Unused child lanes reference the dummy slot behind a box at 1e30.
void setChild4(float4* rec, int lane, const Box& b, uint32_t ref) {
    float* f = reinterpret_cast<float*>(rec);
    for (int a = 0; a < 3; ++a) {
        f[(2 * a) * 4 + lane] = b.mn[a];
        f[(2 * a + 1) * 4 + lane] = b.mx[a];
    }
    reinterpret_cast<uint32_t*>(rec + 6)[lane] = ref;
}

// Collapses the binary tree under `t` (an interior node) into 4-wide nodes:
// a node's children are the binary subtrees reached by repeatedly opening the
// interior child of largest surface area until there are four.
uint32_t flatten4(const TNode* t, std::vector<float4>& nodes, uint32_t dummyLeaf, int depth, int& maxDepth) {
    maxDepth = std::max(maxDepth, depth);
    std::vector<const TNode*> kids = {t->l.get(), t->r.get()};
    while (kids.size() < 4) {
        int best = -1;
        float area = -1.0f;
        for (int i = 0; i < (int)kids.size(); ++i)
            if (kids[i]->l && kids[i]->box.halfArea() > area) {
                area = kids[i]->box.halfArea();
                best = i;
            }
        if (best < 0) break;
        const TNode* open = kids[best];
        kids[best] = open->l.get();
        kids.insert(kids.begin() + best + 1, open->r.get());
    }
    uint32_t idx = (uint32_t)(nodes.size() / 8);
    nodes.resize(nodes.size() + 8);
    uint32_t refs[4];
    for (size_t k = 0; k < kids.size(); ++k)
        refs[k] = kids[k]->l ? flatten4(kids[k], nodes, dummyLeaf, depth + 1, maxDepth)
                             : (kLeaf | (kids[k]->first << 3) | (kids[k]->count - 1u));
    float4* rec = &nodes[8 * (size_t)idx];
    Box far;
    for (int a = 0; a < 3; ++a) far.mn[a] = far.mx[a] = 1e30f;
    for (int k = 0; k < 4; ++k) {
        if (k < (int)kids.size())
            setChild4(rec, k, kids[k]->box, refs[k]);
        else
            setChild4(rec, k, far, dummyLeaf);
    }
    rec[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return idx;
}

}  // namespace

// DFS leaf order of the caller's flat BVH (left child first), the tie order of
// the reference's closest-hit loop.  Triangles no leaf reaches get kNoSlot:
// the reference never intersects them.  Returns false with `err` set when the
// tree is malformed (child or leaf range out of bounds, or a cycle).
bool referenceSlots(const dk_scene* sc, std::vector<uint32_t>& slotOfTri, std::string& err) {
    slotOfTri.assign(sc->triangle_count, kNoSlot);
    if (sc->node_count == 0) {  // linear fallback order (PathTrace.metal:3264-3290)
        for (uint32_t i = 0; i < sc->triangle_count; ++i) slotOfTri[i] = i;
        return true;
    }
    std::vector<uint32_t> stack = {0u};
    uint64_t visits = 0, slot = 0;
    while (!stack.empty()) {
        uint32_t ni = stack.back();
        stack.pop_back();
        if (ni >= sc->node_count) {
            err = "BVH child index out of range";
            return false;
        }
        if (++visits > 2ull * sc->node_count + 2) {
            err = "BVH contains a cycle";
            return false;
        }
        const dk_bvh_node& n = sc->nodes[ni];
        if (n.metadata.w > 0) {
            if ((uint64_t)n.metadata.z + n.metadata.w > sc->primitive_index_count) {
                err = "BVH leaf range out of range";
                return false;
            }
            for (uint32_t k = 0; k < n.metadata.w; ++k) {
                uint32_t t = sc->primitive_indices[n.metadata.z + k];
                if (t < sc->triangle_count && slotOfTri[t] == kNoSlot) slotOfTri[t] = (uint32_t)slot;
                ++slot;
            }
        } else {
            stack.push_back(n.metadata.y);
            stack.push_back(n.metadata.x);
        }
    }
    return true;
}

// Binned-SAH traversal tree over every triangle that has a slot.
int buildSahTraversal(const dk_scene* sc, const std::vector<uint32_t>& slotOfTri,
                      const std::vector<uint8_t>& opaque, std::vector<float4>& nodes, std::vector<float4>& isect,
                      std::string& err) {
    std::vector<Prim> prims;
    prims.reserve(sc->triangle_count);
    for (uint32_t i = 0; i < sc->triangle_count; ++i) {
        if (slotOfTri[i] == kNoSlot) continue;
        const dk_triangle& t = sc->triangles[i];
        Prim p;
        const float* v[3] = {&t.v0.x, &t.v1.x, &t.v2.x};
        for (int a = 0; a < 3; ++a) {
            p.mn[a] = std::fmin(std::fmin(v[0][a], v[1][a]), v[2][a]);
            p.mx[a] = std::fmax(std::fmax(v[0][a], v[1][a]), v[2][a]);
            p.c[a] = 0.5f * (p.mn[a] + p.mx[a]);
        }
        p.tri = i;
        prims.push_back(p);
    }
    nodes.clear();
    isect.clear();
    const uint32_t n = (uint32_t)prims.size();
    if (n >= (1u << 28)) {
        err = "too many triangles for the traversal encoding";
        return DK_ERROR_INVALID_SCENE;
    }
    if (n == 0) return DK_OK;
    std::unique_ptr<TNode> root = build(prims.data(), 0, n, 0);
    isect.resize(3 * (size_t)(n + 1));
    for (uint32_t s = 0; s < n; ++s) {
        const dk_triangle& t = sc->triangles[prims[s].tri];
        isect[3 * (size_t)s + 0] = make_float4(t.v0.x, t.v0.y, t.v0.z, asFloat(slotOfTri[prims[s].tri]));
        isect[3 * (size_t)s + 1] = make_float4(t.v1.x - t.v0.x, t.v1.y - t.v0.y, t.v1.z - t.v0.z, asFloat(prims[s].tri));
        uint32_t mid = std::min(std::min(t.material_id, sc->material_count - 1u), 255u);
        uint32_t flags = (opaque[prims[s].tri] ? 1u : 0u) | (mid << 8);
        isect[3 * (size_t)s + 2] = make_float4(t.v2.x - t.v0.x, t.v2.y - t.v0.y, t.v2.z - t.v0.z, asFloat(flags));
    }
    isect[3 * (size_t)n + 0] = make_float4(0, 0, 0, asFloat(0xffffffffu));  // dummy slot (degenerate)
    isect[3 * (size_t)n + 1] = make_float4(0, 0, 0, asFloat(0u));
    isect[3 * (size_t)n + 2] = make_float4(0, 0, 0, 0);
    int maxDepth = 0;
    const uint32_t dummyLeaf = kLeaf | (n << 3);
    if (!root->l) {  // single leaf: a root with the leaf and three dummy children
        nodes.resize(8);
        Box far;
        for (int a = 0; a < 3; ++a) far.mn[a] = far.mx[a] = 1e30f;
        setChild4(&nodes[0], 0, root->box, kLeaf | (0u << 3) | (root->count - 1u));
        for (int k = 1; k < 4; ++k) setChild4(&nodes[0], k, far, dummyLeaf);
        nodes[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return DK_OK;
    }
    flatten4(root.get(), nodes, dummyLeaf, 0, maxDepth);
    // Each level pushes at most three siblings on the 64-entry traversal stack.
    if (3 * (maxDepth + 1) + 1 > 64) {
        err = "traversal BVH deeper than the 64-entry stack";
        return DK_ERROR_INVALID_SCENE;
    }
    return DK_OK;
}

}  // namespace dk
