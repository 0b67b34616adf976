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
// Output layouts (`width`):
// * 4 (the default): the binary SAH tree (leaves of <= 8 triangles) collapsed
//   into 4-wide nodes of 8 x float4 (the x, y, z slabs of four children, one
//   lane each, and the four child references: interior index, or 0x80000000 |
//   first << 3 | (count - 1) for a leaf); one dummy slot at the end;
// * 8: the binary SAH tree (leaves of <= 4 triangles) collapsed into 8-wide
//   nodes of 5 x 16 bytes with child boxes quantised to 8 bits per bound
//   (record layout at `Quantizer` below; the compressed wide BVH of Ylitie,
//   Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through
//   Compressed Wide BVHs", HPG 2017, with an encoding of this file's own), the
//   slots of a node's leaves consecutive.
// Both: 3 x float4 per leaf slot: (v0, reference slot), (v1 - v0, triangle
// index), (v2 - v0, flags: bit 0 = blocks shadow rays, bits 8..15 material
// ID).
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <deque>
#include <mutex>
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
#ifndef DK_SAH_BINS
#define DK_SAH_BINS 32
#endif
#ifndef DK_SAH_NODE_COST
#define DK_SAH_NODE_COST 1.0f
#endif
#ifndef DK_SAH_MAX_LEAF
#define DK_SAH_MAX_LEAF 8  // <= 8: a 4-wide child reference holds count - 1 in 3 bits
#endif
static_assert(DK_SAH_MAX_LEAF >= 1 && DK_SAH_MAX_LEAF <= 8, "leaf size must fit the child encoding");
constexpr int kBins = DK_SAH_BINS;
constexpr float kNodeCost = DK_SAH_NODE_COST;  // traversal step cost in triangle tests

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
    TNode* l = nullptr;
    TNode* r = nullptr;
    uint32_t first = 0, count = 0;  // triangle range of the subtree (in SAH order)
    uint32_t wide = 0;              // 4-wide nodes of the collapsed subtree rooted here
};

// Nodes come from per-task chunked arenas (one heap allocation per 16K nodes,
// not per node); the arenas live until the wide tree has been emitted.
class NodeArena {
  public:
    TNode* alloc() {
        if (chunks_.empty() || used_ == kChunk) {
            chunks_.emplace_back(new TNode[kChunk]);
            used_ = 0;
        }
        return &chunks_.back()[used_++];
    }

  private:
    static constexpr size_t kChunk = 16384;
    std::vector<std::unique_ptr<TNode[]>> chunks_;
    size_t used_ = 0;
};

struct Arenas {
    std::mutex m;
    std::deque<NodeArena> list;
    NodeArena& make() {
        std::lock_guard<std::mutex> g(m);
        list.emplace_back();
        return list.back();
    }
};

// Per-axis bins of one node: the union of the primitive boxes and the count,
// for each of kBins centroid bins.  Only the counts are initialised: a bin's
// box is set by its first primitive and read only while its count is
// non-zero (an empty bin is the identity of the union), so a small node does
// not pay for the whole table.
struct AxisBins {
    Box box[kBins];
    uint32_t cnt[kBins];
};

struct NodeBins {
    AxisBins axis[3];
    NodeBins() {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < kBins; ++b) axis[a].cnt[b] = 0;
    }
    void add(int a, int b, const Prim& q) {
        AxisBins& ab = axis[a];
        if (ab.cnt[b]++ == 0) {
            for (int k = 0; k < 3; ++k) {
                ab.box[b].mn[k] = q.mn[k];
                ab.box[b].mx[k] = q.mx[k];
            }
        } else {
            ab.box[b].grow(q.mn, q.mx);
        }
    }
    void merge(const NodeBins& o) {
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < kBins; ++b) {
                if (o.axis[a].cnt[b] == 0) continue;
                if (axis[a].cnt[b] == 0)
                    axis[a].box[b] = o.axis[a].box[b];
                else
                    axis[a].box[b].grow(o.axis[a].box[b]);
                axis[a].cnt[b] += o.axis[a].cnt[b];
            }
    }
};

inline int binOf(float c, float lo, float scale) { return std::min(kBins - 1, (int)((c - lo) * scale)); }

void binRange(const Prim* p, uint32_t begin, uint32_t end, const Box& cb, const float* scale, const bool* live,
              NodeBins& nb) {
    for (uint32_t i = begin; i < end; ++i)
        for (int a = 0; a < 3; ++a)
            if (live[a]) nb.add(a, binOf(p[i].c[a], cb.mn[a], scale[a]), p[i]);
}

// The union of the centroids of [begin, end) (several threads for a long range).
void centroidBounds(const Prim* p, uint32_t begin, uint32_t end, Box& out) {
    const uint32_t n = end - begin;
    if (n < (1u << 18)) {
        for (uint32_t i = begin; i < end; ++i) out.grow(p[i].c, p[i].c);
        return;
    }
    const uint32_t parts = std::min<uint32_t>(16, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<Box> part(parts);
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < parts; ++t)
        pool.emplace_back([&, t] {
            uint32_t b0 = begin + (uint32_t)((uint64_t)n * t / parts), b1 = begin + (uint32_t)((uint64_t)n * (t + 1) / parts);
            for (uint32_t i = b0; i < b1; ++i) part[t].grow(p[i].c, p[i].c);
        });
    for (auto& th : pool) th.join();
    for (const Box& b : part) out.grow(b);
}

// Binned SAH (traversal cost kNodeCost, intersection cost 1) over the node's
// primitives [first, first + n), whose box and centroid box are given.
// Children inherit their boxes from the chosen split's bins (unions, exact);
// their centroid boxes come from one pass over the partitioned primitives.
TNode* build(Prim* p, uint32_t first, uint32_t n, int depth, uint32_t maxLeaf, const Box& box, const Box& cb,
             Arenas& arenas, NodeArena& arena) {
    TNode* node = arena.alloc();
    node->box = box;
    node->first = first;
    node->count = n;
    if (n == 1) return node;
    float scale[3];
    bool live[3];
    for (int a = 0; a < 3; ++a) {
        float ext = cb.mx[a] - cb.mn[a];
        live[a] = ext > 0.0f;
        scale[a] = live[a] ? (float)kBins / ext : 0.0f;
    }
    NodeBins nb;
    const uint32_t kParallelBins = 1u << 18;
    if (n >= kParallelBins) {  // large node: bin slices on several threads, merge the unions
        const uint32_t parts = std::min<uint32_t>(16, std::max(1u, std::thread::hardware_concurrency()));
        std::vector<NodeBins> partial(parts);
        std::vector<std::thread> pool;
        for (uint32_t t = 0; t < parts; ++t)
            pool.emplace_back([&, t] {
                uint32_t b0 = first + (uint32_t)((uint64_t)n * t / parts), b1 = first + (uint32_t)((uint64_t)n * (t + 1) / parts);
                binRange(p, b0, b1, cb, scale, live, partial[t]);
            });
        for (auto& th : pool) th.join();
        for (uint32_t t = 0; t < parts; ++t) nb.merge(partial[t]);
    } else {
        binRange(p, first, first + n, cb, scale, live, nb);
    }
    // The sweeps visit the non-empty bins only: the cost of a split after an
    // empty bin equals the cost after the last non-empty bin before it, and
    // the strict `<` keeps that earlier bin, which is the split the full
    // 32-bin sweep selects.
    float bestCost = FLT_MAX;
    int bestAxis = -1, bestSplit = -1;
    for (int a = 0; a < 3; ++a) {
        if (!live[a]) continue;
        const AxisBins& ab = nb.axis[a];
        int nz[kBins], m = 0;
        for (int b = 0; b < kBins; ++b)
            if (ab.cnt[b]) nz[m++] = b;
        float rightArea[kBins];
        uint32_t rightCount[kBins];
        Box acc;
        uint32_t cnt = 0;
        for (int k = m - 1; k > 0; --k) {  // right side from the k-th non-empty bin on
            acc.grow(ab.box[nz[k]]);
            cnt += ab.cnt[nz[k]];
            rightArea[k] = acc.halfArea();
            rightCount[k] = cnt;
        }
        acc = Box();
        cnt = 0;
        for (int k = 0; k + 1 < m; ++k) {
            acc.grow(ab.box[nz[k]]);
            cnt += ab.cnt[nz[k]];
            float cost = acc.halfArea() * (float)cnt + rightArea[k + 1] * (float)rightCount[k + 1];
            if (cost < bestCost) {
                bestCost = cost;
                bestAxis = a;
                bestSplit = nz[k];
            }
        }
    }
    float nodeArea = box.halfArea();
    float splitCost = kNodeCost + (nodeArea > 0.0f ? bestCost / nodeArea : 0.0f);
    if (n <= maxLeaf && (bestAxis < 0 || (float)n <= splitCost)) return node;
    uint32_t mid;
    Box lb, rb, lc, rc;
    bool haveBoxes = false;
    if (bestAxis >= 0) {
        const int a = bestAxis, sp = bestSplit;
        const float lo = cb.mn[a], sc = scale[a];
        Prim* m = std::partition(p + first, p + first + n, [=](const Prim& q) { return binOf(q.c[a], lo, sc) <= sp; });
        mid = (uint32_t)(m - p);
        if (mid != first && mid != first + n) {
            const AxisBins& ab = nb.axis[a];
            for (int b = 0; b < kBins; ++b) {
                if (!ab.cnt[b]) continue;
                (b <= sp ? lb : rb).grow(ab.box[b]);
            }
            centroidBounds(p, first, mid, lc);
            centroidBounds(p, mid, first + n, rc);
            haveBoxes = true;
        } else {
            mid = first + n / 2;
        }
    } else {  // coincident centroids: split the range in half
        mid = first + n / 2;
    }
    if (!haveBoxes) {  // a range split: boxes of the two halves
        for (uint32_t i = first; i < mid; ++i) {
            lb.grow(p[i].mn, p[i].mx);
            lc.grow(p[i].c, p[i].c);
        }
        for (uint32_t i = mid; i < first + n; ++i) {
            rb.grow(p[i].mn, p[i].mx);
            rc.grow(p[i].c, p[i].c);
        }
    }
    if (n > 16384 && depth < 9) {
        NodeArena& other = arenas.make();
        auto fut = std::async(std::launch::async, [&, first, mid, depth, maxLeaf] {
            return build(p, first, mid - first, depth + 1, maxLeaf, lb, lc, arenas, other);
        });
        node->r = build(p, mid, first + n - mid, depth + 1, maxLeaf, rb, rc, arenas, arena);
        node->l = fut.get();
    } else {
        node->l = build(p, first, mid - first, depth + 1, maxLeaf, lb, lc, arenas, arena);
        node->r = build(p, mid, first + n - mid, depth + 1, maxLeaf, rb, rc, arenas, arena);
    }
    return node;
}

// The tree over all primitives; the root's boxes from a parallel pass.
TNode* buildTree(std::vector<Prim>& prims, uint32_t maxLeaf, Arenas& arenas) {
    const uint32_t n = (uint32_t)prims.size();
    const uint32_t parts = std::min<uint32_t>(16, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<Box> pb(parts), pc(parts);
    std::vector<std::thread> pool;
    for (uint32_t t = 0; t < parts; ++t)
        pool.emplace_back([&, t] {
            uint32_t b0 = (uint32_t)((uint64_t)n * t / parts), b1 = (uint32_t)((uint64_t)n * (t + 1) / parts);
            for (uint32_t i = b0; i < b1; ++i) {
                pb[t].grow(prims[i].mn, prims[i].mx);
                pc[t].grow(prims[i].c, prims[i].c);
            }
        });
    for (auto& th : pool) th.join();
    Box box, cb;
    for (uint32_t t = 0; t < parts; ++t) {
        box.grow(pb[t]);
        cb.grow(pc[t]);
    }
    return build(prims.data(), 0, n, 0, maxLeaf, box, cb, arenas, arenas.make());
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

// The children of the 4-wide node at interior node `t`: the binary subtrees
// reached by repeatedly opening the interior child of largest surface area
// until there are four.
int collapse4(const TNode* t, const TNode* kids[4]) {
    int k = 2;
    kids[0] = t->l;
    kids[1] = t->r;
    while (k < 4) {
        int best = -1;
        float area = -1.0f;
        for (int i = 0; i < k; ++i)
            if (kids[i]->l && kids[i]->box.halfArea() > area) {
                area = kids[i]->box.halfArea();
                best = i;
            }
        if (best < 0) break;
        const TNode* open = kids[best];
        for (int i = k; i > best + 1; --i) kids[i] = kids[i - 1];
        kids[best] = open->l;
        kids[best + 1] = open->r;
        ++k;
    }
    return k;
}

// Counts the 4-wide nodes of every collapsed subtree (TNode::wide) and the
// tree depth; large subtrees on other threads.
uint32_t count4(TNode* t, int depth, int& maxDepth) {
    maxDepth = std::max(maxDepth, depth);
    const TNode* kids[4];
    const int k = collapse4(t, kids);
    uint32_t total = 1;
    std::vector<std::future<std::pair<uint32_t, int>>> forks;
    for (int i = 0; i < k; ++i) {
        if (!kids[i]->l) continue;
        TNode* c = const_cast<TNode*>(kids[i]);
        if (depth < 5 && c->count > 65536) {
            forks.push_back(std::async(std::launch::async, [c, depth] {
                int md = 0;
                uint32_t w = count4(c, depth + 1, md);
                return std::make_pair(w, md);
            }));
        } else {
            total += count4(c, depth + 1, maxDepth);
        }
    }
    for (auto& f : forks) {
        auto r = f.get();
        total += r.first;
        maxDepth = std::max(maxDepth, r.second);
    }
    t->wide = total;
    return total;
}

// Writes the 4-wide node of `t` at index `idx` and its subtree after it in
// depth-first order (interior children's subtrees in child order), into the
// pre-sized `nodes`; large subtrees on other threads.
void emit4(const TNode* t, uint32_t idx, float4* nodes, uint32_t dummyLeaf, int depth) {
    const TNode* kids[4];
    const int k = collapse4(t, kids);
    uint32_t refs[4], next = idx + 1;
    for (int i = 0; i < k; ++i) {
        if (kids[i]->l) {
            refs[i] = next;
            next += kids[i]->wide;
        } else {
            refs[i] = kLeaf | (kids[i]->first << 3) | (kids[i]->count - 1u);
        }
    }
    float4* rec = nodes + 8 * (size_t)idx;
    Box far;
    for (int a = 0; a < 3; ++a) far.mn[a] = far.mx[a] = 1e30f;
    for (int i = 0; i < 4; ++i) {
        if (i < k)
            setChild4(rec, i, kids[i]->box, refs[i]);
        else
            setChild4(rec, i, far, dummyLeaf);
    }
    rec[7] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    std::vector<std::future<void>> forks;
    for (int i = 0; i < k; ++i) {
        if (!kids[i]->l) continue;
        if (depth < 5 && kids[i]->wide > 8192)
            forks.push_back(std::async(std::launch::async, [=] { emit4(kids[i], refs[i], nodes, dummyLeaf, depth + 1); }));
        else
            emit4(kids[i], refs[i], nodes, dummyLeaf, depth + 1);
    }
    for (auto& f : forks) f.get();
}

// 8-wide node record (5 x 16 bytes):
//   word 0: origin p (3 x f32: the node box minimum), then one byte each of
//           the biased exponents of the x, y, z quantisation steps and the
//           mask of interior children (bit = slot);
//   word 1: index of the first interior child node, index of the first leaf
//           slot, and one byte per child slot: (count << 5) | offset of the
//           leaf's triangles from the first leaf slot (0 for interior and
//           empty slots);
//   words 2-4: per child slot, 8-bit box bounds lo.x, lo.y, lo.z, hi.x, hi.y,
//           hi.z (8 bytes each, slot s in byte s), i.e. the box
//           p + q * 2^(E - 127) per axis, rounded outwards.
// Interior children are stored consecutively from the first child index in
// slot order, and so are the leaves' triangles from the first leaf slot.
// The child in slot s is the one lying furthest towards the box corner s (bit
// a of s set = high side on axis a), so a ray whose direction signs form s
// meets slot s first; the traversal visits slots in the order (slot ^ s).
struct Quantizer {
    float p[3];
    double e[3];
    uint32_t E[3];
    explicit Quantizer(const Box& b) {
        for (int a = 0; a < 3; ++a) {
            p[a] = b.mn[a];
            double ext = (double)b.mx[a] - (double)b.mn[a];
            int k = -126;
            if (ext > 0.0) {
                k = (int)std::ceil(std::log2(ext / 255.0));
                while (std::ldexp(1.0, k) * 255.0 <= ext) ++k;  // strictly above: the top plane keeps a margin
                while (k > -126 && std::ldexp(1.0, k - 1) * 255.0 > ext) --k;
            }
            k = std::max(-126, std::min(127, k));
            E[a] = (uint32_t)(k + 127);
            e[a] = std::ldexp(1.0, k);
        }
    }
    // Outward-rounded bounds of `b`; a bound that falls exactly on a grid
    // plane is moved one step out (except the node's own minimum plane, which
    // the traversal evaluates exactly), so child boxes keep a margin.
    void quantize(const Box& b, int a, uint32_t& lo, uint32_t& hi) const {
        double rl = ((double)b.mn[a] - (double)p[a]) / e[a];
        double rh = ((double)b.mx[a] - (double)p[a]) / e[a];
        double ql = std::floor(rl), qh = std::ceil(rh);
        if (ql == rl && ql > 0.0) ql -= 1.0;
        if (qh == rh && qh < 255.0) qh += 1.0;
        lo = (uint32_t)std::max(0.0, std::min(255.0, ql));
        hi = (uint32_t)std::max(0.0, std::min(255.0, qh));
    }
};

// A leaf of the 8-wide tree: a binary leaf, or a subtree of at most
// DK_WIDE_LEAF_MERGE triangles (consecutive in SAH order; at most 4).
// Merging fills the nodes but tests more triangles per ray; the default
// keeps the SAH leaves.
#ifndef DK_WIDE_LEAF_MERGE
#define DK_WIDE_LEAF_MERGE 1
#endif
inline bool wideLeaf(const TNode* t) { return !t->l || t->count <= DK_WIDE_LEAF_MERGE; }

struct Wide8Builder {
    const std::vector<Prim>& prims;   // SAH order: leaf ranges index it
    const dk_scene* sc;
    const std::vector<uint32_t>& slotOfTri;
    const std::vector<uint8_t>& opaque;
    std::vector<float4>& nodes;       // 5 x float4 per node
    std::vector<float4>& isect;       // 3 x float4 per leaf slot
    int maxDepth = 0;

    uint32_t appendTriangles(const TNode* leaf) {
        uint32_t first = (uint32_t)(isect.size() / 3);
        for (uint32_t k = leaf->first; k < leaf->first + leaf->count; ++k) {
            uint32_t tri = prims[k].tri;
            const dk_triangle& t = sc->triangles[tri];
            uint32_t mid = std::min(std::min(t.material_id, sc->material_count - 1u), 255u);
            uint32_t flags = (opaque[tri] ? 1u : 0u) | (mid << 8);
            isect.push_back(make_float4(t.v0.x, t.v0.y, t.v0.z, asFloat(slotOfTri[tri])));
            isect.push_back(make_float4(t.v1.x - t.v0.x, t.v1.y - t.v0.y, t.v1.z - t.v0.z, asFloat(tri)));
            isect.push_back(make_float4(t.v2.x - t.v0.x, t.v2.y - t.v0.y, t.v2.z - t.v0.z, asFloat(flags)));
        }
        return first;
    }

    // Children of interior node `t`: binary subtrees reached by repeatedly
    // opening the interior child of largest surface area, up to eight.
    static std::vector<const TNode*> collapse(const TNode* t) {
        if (wideLeaf(t)) return {t};  // a single-leaf tree: the root holds the leaf
        std::vector<const TNode*> kids = {t->l, t->r};
        while (kids.size() < 8) {
            int best = -1;
            float area = -1.0f;
            for (int i = 0; i < (int)kids.size(); ++i)
                if (!wideLeaf(kids[i]) && kids[i]->box.halfArea() > area) {
                    area = kids[i]->box.halfArea();
                    best = i;
                }
            if (best < 0) break;
            const TNode* open = kids[best];
            kids[best] = open->l;
            kids.push_back(open->r);
        }
        return kids;
    }

    // Slot of every child: greedy assignment of (corner, child) pairs in
    // decreasing order of how far the child's centre lies towards the corner.
    static void assignSlots(const Box& nb, const std::vector<const TNode*>& kids, const TNode* slot[8]) {
        for (int s = 0; s < 8; ++s) slot[s] = nullptr;
        struct Cand { float score; int s, k; };
        std::vector<Cand> cand;
        float cn[3];
        for (int a = 0; a < 3; ++a) cn[a] = 0.5f * (nb.mn[a] + nb.mx[a]);
        for (int k = 0; k < (int)kids.size(); ++k) {
            float c[3];
            for (int a = 0; a < 3; ++a) c[a] = 0.5f * (kids[k]->box.mn[a] + kids[k]->box.mx[a]) - cn[a];
            for (int s = 0; s < 8; ++s) {
                float sc = 0.0f;
                for (int a = 0; a < 3; ++a) sc += ((s >> a) & 1) ? c[a] : -c[a];
                cand.push_back({sc, s, k});
            }
        }
        std::stable_sort(cand.begin(), cand.end(), [](const Cand& x, const Cand& y) { return x.score > y.score; });
        bool used[8] = {};
        for (const Cand& c : cand) {
            if (slot[c.s] || used[c.k]) continue;
            slot[c.s] = kids[c.k];
            used[c.k] = true;
        }
    }

    // Writes the record of interior node `t` at index `idx`, then its subtree.
    void emit(const TNode* t, uint32_t idx, int depth) {
        maxDepth = std::max(maxDepth, depth);
        std::vector<const TNode*> kids = collapse(t);
        const TNode* slot[8];
        assignSlots(t->box, kids, slot);
        Quantizer qz(t->box);
        uint32_t imask = 0, nInterior = 0;
        for (int s = 0; s < 8; ++s)
            if (slot[s] && !wideLeaf(slot[s])) {
                imask |= 1u << s;
                ++nInterior;
            }
        const uint32_t childBase = (uint32_t)(nodes.size() / 5);
        nodes.resize(nodes.size() + 5 * (size_t)nInterior);
        const uint32_t triBase = (uint32_t)(isect.size() / 3);
        uint8_t meta[8] = {}, q[6][8] = {};
        for (int s = 0; s < 8; ++s) {
            const TNode* c = slot[s];
            if (!c) continue;
            for (int a = 0; a < 3; ++a) {
                uint32_t lo, hi;
                qz.quantize(c->box, a, lo, hi);
                q[a][s] = (uint8_t)lo;
                q[3 + a][s] = (uint8_t)hi;
            }
            if (wideLeaf(c)) {
                uint32_t first = appendTriangles(c);
                meta[s] = (uint8_t)((c->count << 5) | (first - triBase));
            }
        }
        uint32_t w[20];
        std::memcpy(&w[0], &qz.p[0], 4);
        std::memcpy(&w[1], &qz.p[1], 4);
        std::memcpy(&w[2], &qz.p[2], 4);
        w[3] = qz.E[0] | (qz.E[1] << 8) | (qz.E[2] << 16) | (imask << 24);
        w[4] = childBase;
        w[5] = triBase;
        std::memcpy(&w[6], meta, 8);
        std::memcpy(&w[8], q, 48);
        std::memcpy(&nodes[5 * (size_t)idx], w, 80);
        uint32_t j = 0;
        for (int s = 0; s < 8; ++s)
            if (slot[s] && !wideLeaf(slot[s])) emit(slot[s], childBase + j++, depth + 1);
    }
};

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

namespace {
// DK_TRACE_CREATE=1: the traversal build's phases (host wall time) on stderr.
struct BuildTrace {
    bool on;
    std::chrono::steady_clock::time_point t;
    BuildTrace() {
        const char* e = getenv("DK_TRACE_CREATE");
        on = e && e[0] == '1';
        t = std::chrono::steady_clock::now();
    }
    void mark(const char* what) {
        if (!on) return;
        auto now = std::chrono::steady_clock::now();
        fprintf(stderr, "[dk create]   %s %.1f ms\n", what, std::chrono::duration<double, std::milli>(now - t).count());
        t = now;
    }
};
}  // namespace

// Binned-SAH traversal tree over every triangle that has a slot.
int buildSahTraversal(const dk_scene* sc, const std::vector<uint32_t>& slotOfTri,
                      const std::vector<uint8_t>& opaque, int width, std::vector<float4>& nodes,
                      std::vector<float4>& isect, std::string& err) {
    // Primitives of the triangles that have a slot, in triangle order: the
    // slotted triangles are counted per chunk, then every chunk writes its
    // primitives at its offset (several threads).
    BuildTrace trace;
    const uint32_t tc = sc->triangle_count;
    const uint32_t parts = std::min<uint32_t>(16, std::max(1u, std::thread::hardware_concurrency()));
    std::vector<uint32_t> offset(parts + 1, 0);
    auto chunk = [&](uint32_t t, uint32_t& b0, uint32_t& b1) {
        b0 = (uint32_t)((uint64_t)tc * t / parts);
        b1 = (uint32_t)((uint64_t)tc * (t + 1) / parts);
    };
    for (uint32_t t = 0; t < parts; ++t) {
        uint32_t b0, b1;
        chunk(t, b0, b1);
        uint32_t c = 0;
        for (uint32_t i = b0; i < b1; ++i) c += slotOfTri[i] != kNoSlot;
        offset[t + 1] = offset[t] + c;
    }
    std::vector<Prim> prims(offset[parts]);
    {
        std::vector<std::thread> pool;
        for (uint32_t t = 0; t < parts; ++t)
            pool.emplace_back([&, t] {
                uint32_t b0, b1, o = offset[t];
                chunk(t, b0, b1);
                for (uint32_t i = b0; i < b1; ++i) {
                    if (slotOfTri[i] == kNoSlot) continue;
                    const dk_triangle& tr = sc->triangles[i];
                    Prim& q = prims[o++];
                    const float* v[3] = {&tr.v0.x, &tr.v1.x, &tr.v2.x};
                    for (int a = 0; a < 3; ++a) {
                        q.mn[a] = std::fmin(std::fmin(v[0][a], v[1][a]), v[2][a]);
                        q.mx[a] = std::fmax(std::fmax(v[0][a], v[1][a]), v[2][a]);
                        q.c[a] = 0.5f * (q.mn[a] + q.mx[a]);
                    }
                    q.tri = i;
                }
            });
        for (auto& th : pool) th.join();
    }
    trace.mark("primitive records");
    nodes.clear();
    isect.clear();
    const uint32_t n = (uint32_t)prims.size();
    if (n >= (1u << 28)) {
        err = "too many triangles for the traversal encoding";
        return DK_ERROR_INVALID_SCENE;
    }
    if (n == 0) return DK_OK;
    if (width == 8) {
        // Leaves of <= 4 triangles: eight of them fill a node's 32-bit slot mask.
        Arenas arenas;
        TNode* root = buildTree(prims, 4, arenas);
        isect.reserve(3 * (size_t)n);
        nodes.resize(5);
        Wide8Builder wb{prims, sc, slotOfTri, opaque, nodes, isect};
        wb.emit(root, 0, 0);
        // Each node visit pushes at most one group of siblings.
        if (wb.maxDepth + 1 > (int)kTraversalStack) {
            err = "traversal BVH deeper than the traversal stack";
            return DK_ERROR_INVALID_SCENE;
        }
        return DK_OK;
    }
    Arenas arenas;
    TNode* root = buildTree(prims, DK_SAH_MAX_LEAF, arenas);
    trace.mark("binned SAH tree");
    // The leaf slots in SAH order, filled by several threads while this
    // thread collapses the tree (the two are independent).
    isect.resize(3 * (size_t)(n + 1));
    auto fillSlots = [&](uint32_t b0, uint32_t b1) {
        for (uint32_t s = b0; s < b1; ++s) {
            const dk_triangle& t = sc->triangles[prims[s].tri];
            isect[3 * (size_t)s + 0] = make_float4(t.v0.x, t.v0.y, t.v0.z, asFloat(slotOfTri[prims[s].tri]));
            isect[3 * (size_t)s + 1] =
                make_float4(t.v1.x - t.v0.x, t.v1.y - t.v0.y, t.v1.z - t.v0.z, asFloat(prims[s].tri));
            uint32_t mid = std::min(std::min(t.material_id, sc->material_count - 1u), 255u);
            uint32_t flags = (opaque[prims[s].tri] ? 1u : 0u) | (mid << 8);
            isect[3 * (size_t)s + 2] = make_float4(t.v2.x - t.v0.x, t.v2.y - t.v0.y, t.v2.z - t.v0.z, asFloat(flags));
        }
    };
    std::vector<std::thread> fill;
    for (uint32_t t = 0; t < parts; ++t)
        fill.emplace_back(fillSlots, (uint32_t)((uint64_t)n * t / parts), (uint32_t)((uint64_t)n * (t + 1) / parts));
    struct Join {
        std::vector<std::thread>& v;
        ~Join() {
            for (auto& th : v) th.join();
        }
    } join{fill};
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
    const uint32_t wideNodes = count4(root, 0, maxDepth);
    nodes.resize(8 * (size_t)wideNodes);
    emit4(root, 0, nodes.data(), dummyLeaf, 0);
    trace.mark("4-wide collapse");
    // Each level pushes at most three siblings on the 64-entry traversal stack.
    if (3 * (maxDepth + 1) + 1 > 64) {
        err = "traversal BVH deeper than the 64-entry stack";
        return DK_ERROR_INVALID_SCENE;
    }
    return DK_OK;
}

}  // namespace dk
