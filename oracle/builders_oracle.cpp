// Test infrastructure: the CPU oracle for the scene-compile step in front of
// the path tracer.  Only tests/, __graft_entry__.smoke() and bench.py's
// cpu_baseline leg may use anything under oracle/.
//
// Plain restatements of the reference's Swift host builders, in the reference's
// FP32 arithmetic:
//   * BVHBuilder.build + BVHFlattener.flatten
//     (Sources/DenrimRendererKit/Acceleration/BVHBuilder.swift:7-135,
//      FlatBVH.swift:13-32, BVH.swift:4-31)
//   * lightRecordsAndTaggedTriangles and environmentSamples
//     (Sources/DenrimRendererKit/Acceleration/LightingGPUEncoding.swift:5-135)
// Swift's `sort` is not documented as stable; this restatement uses a stable
// sort, which defines "reference node order" for ties in the centroid key.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/denrim_cuda.h"

namespace {

struct F3 { float x, y, z; };
struct Box { F3 mn, mx; };

static inline float axisOf(const F3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
static inline F3 fmin3(F3 a, F3 b) { return {std::fmin(a.x, b.x), std::fmin(a.y, b.y), std::fmin(a.z, b.z)}; }
static inline F3 fmax3(F3 a, F3 b) { return {std::fmax(a.x, b.x), std::fmax(a.y, b.y), std::fmax(a.z, b.z)}; }
// AABB.empty / include: BVH.swift:8-31
static inline Box emptyBox() { return {{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}}; }
static inline void includePoint(Box& b, F3 p) { b.mn = fmin3(b.mn, p); b.mx = fmax3(b.mx, p); }
static inline void includeBox(Box& b, const Box& o) { includePoint(b, o.mn); includePoint(b, o.mx); }
static inline F3 centroid(const Box& b) {
    return {(b.mn.x + b.mx.x) * 0.5f, (b.mn.y + b.mx.y) * 0.5f, (b.mn.z + b.mx.z) * 0.5f};
}
// largestAxis: BVHBuilder.swift:126-134
static inline int largestAxis(F3 e) {
    if (e.x >= e.y && e.x >= e.z) return 0;
    if (e.y >= e.z) return 1;
    return 2;
}

struct Node { Box b; int left, right, first, count; };

struct Builder {
    const std::vector<Box>* prim;
    std::vector<uint32_t>* idx;
    std::vector<Node>* nodes;
    uint32_t maxLeaf;
    // buildNode: BVHBuilder.swift:34-92 (pre-order numbering, leaf when
    // count <= max(1, maxLeafPrimitiveCount), median split after a sort on the
    // centroid of the largest centroid-extent axis).
    int build(uint32_t lo, uint32_t hi) {
        int nodeIndex = (int)nodes->size();
        Box bounds = emptyBox();
        for (uint32_t i = lo; i < hi; ++i) includeBox(bounds, (*prim)[(*idx)[i]]);
        nodes->push_back({bounds, -1, -1, (int)lo, (int)(hi - lo)});
        uint32_t count = hi - lo;
        if (!(count > std::max(1u, maxLeaf))) return nodeIndex;
        Box cb = emptyBox();
        for (uint32_t i = lo; i < hi; ++i) includePoint(cb, centroid((*prim)[(*idx)[i]]));
        F3 ext = {cb.mx.x - cb.mn.x, cb.mx.y - cb.mn.y, cb.mx.z - cb.mn.z};
        int axis = largestAxis(ext);
        const std::vector<Box>& P = *prim;
        std::stable_sort(idx->begin() + lo, idx->begin() + hi, [&](uint32_t l, uint32_t r) {
            return axisOf(centroid(P[l]), axis) < axisOf(centroid(P[r]), axis);
        });
        uint32_t mid = lo + count / 2;
        int left = build(lo, mid);
        int right = build(mid, hi);
        (*nodes)[nodeIndex] = {bounds, left, right, -1, 0};
        return nodeIndex;
    }
};

static inline F3 ld(const dk_float4& f) { return {f.x, f.y, f.z}; }
static inline F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline F3 crs(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
static inline float dt(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float lum(F3 v) { return dt(v, {0.2126f, 0.7152f, 0.0722f}); }

}  // namespace

extern "C" {

// BVHBuilder(maxLeafPrimitiveCount:).build(triangles:) then BVHFlattener.flatten.
// nodes_out must hold 2*n nodes; returns the node count.
uint32_t oracle_build_bvh(const dk_triangle* tris, uint32_t n, uint32_t maxLeaf, dk_bvh_node* nodes_out,
                          uint32_t* prim_out) {
    if (n == 0) return 0;
    std::vector<Box> prim(n);
    for (uint32_t i = 0; i < n; ++i) {  // BVHBuilder.bounds(for:), BVHBuilder.swift:94-100
        Box b = emptyBox();
        includePoint(b, ld(tris[i].v0));
        includePoint(b, ld(tris[i].v1));
        includePoint(b, ld(tris[i].v2));
        prim[i] = b;
    }
    std::vector<uint32_t> idx(n);
    for (uint32_t i = 0; i < n; ++i) idx[i] = i;
    std::vector<Node> nodes;
    nodes.reserve(2 * (size_t)n);
    Builder b{&prim, &idx, &nodes, maxLeaf};
    b.build(0, n);
    for (size_t i = 0; i < nodes.size(); ++i) {  // BVHFlattener.gpuNode, FlatBVH.swift:21-32
        const Node& s = nodes[i];
        dk_bvh_node& d = nodes_out[i];
        d.bounds_min = {s.b.mn.x, s.b.mn.y, s.b.mn.z, 0.0f};
        d.bounds_max = {s.b.mx.x, s.b.mx.y, s.b.mx.z, 0.0f};
        d.metadata = {(uint32_t)std::max(0, s.left), (uint32_t)std::max(0, s.right), (uint32_t)std::max(0, s.first),
                      (uint32_t)std::max(0, s.count)};
    }
    std::memcpy(prim_out, idx.data(), sizeof(uint32_t) * n);
    return (uint32_t)nodes.size();
}

// lightRecordsAndTaggedTriangles: LightingGPUEncoding.swift:5-64.  Tags
// padding2 in place; returns the light count.
uint32_t oracle_build_lights(dk_triangle* tris, uint32_t n, const dk_material* mats, uint32_t materialCount,
                             dk_light_record* out) {
    if (materialCount == 0) return 0;
    struct Cand { uint32_t tri, mat; float area, weight; F3 normal; };
    std::vector<Cand> cands;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t mi = std::min(tris[i].material_id, materialCount - 1);
        const dk_material& m = mats[mi];
        if (!(std::fmax(std::fmax(m.emission.x, m.emission.y), m.emission.z) > 0.0f)) continue;
        F3 a = sub(ld(tris[i].v1), ld(tris[i].v0));
        F3 b = sub(ld(tris[i].v2), ld(tris[i].v0));
        F3 c = crs(a, b);
        float area = std::sqrt(dt(c, c)) * 0.5f;
        if (!(area > 0.0f)) continue;
        float power = lum(ld(m.emission)) * area;
        if (!(power > 0.0f)) continue;
        float len = std::sqrt(dt(c, c));
        float s = 1.0f / len;
        cands.push_back({i, mi, area, power, {c.x * s, c.y * s, c.z * s}});
    }
    float total = 0.0f;
    for (auto& c : cands) total += c.weight;
    if (!(total > 0.0f)) return 0;
    float cumulative = 0.0f;
    for (size_t k = 0; k < cands.size(); ++k) {
        cumulative += cands[k].weight;
        float cdf = k == cands.size() - 1 ? 1.0f : std::fmin(cumulative / total, 1.0f);
        tris[cands[k].tri].padding2 = (uint32_t)(k + 1);
        out[k].triangle_index = cands[k].tri;
        out[k].material_index = cands[k].mat;
        out[k].area = cands[k].area;
        out[k].selection_cdf = cdf;
        out[k].normal = {cands[k].normal.x, cands[k].normal.y, cands[k].normal.z, 0.0f};
    }
    return (uint32_t)cands.size();
}

// environmentSamples: LightingGPUEncoding.swift:66-119 (FP32 running sum).
// Returns the number of entries written (0 when the map has no energy).
uint32_t oracle_build_environment_samples(const dk_float4* px, uint32_t w, uint32_t h, float intensity_,
                                          float maxRadiance_, dk_environment_sample* out) {
    if (w == 0 || h == 0) return 0;
    float intensity = std::fmax(intensity_, 0.0f);
    float maxRadiance = std::fmax(maxRadiance_, 0.0f);
    float dTheta = (float)M_PI / (float)h;
    float dPhi = 2.0f * (float)M_PI / (float)w;
    std::vector<float> weights((size_t)w * h);
    float total = 0.0f;
    for (uint32_t y = 0; y < h; ++y) {
        float theta = ((float)y + 0.5f) * dTheta;
        float solid = std::fmax(std::sin(theta) * dTheta * dPhi, 1e-8f);
        for (uint32_t x = 0; x < w; ++x) {
            const dk_float4& t = px[(size_t)y * w + x];
            F3 c = {t.x * intensity, t.y * intensity, t.z * intensity};
            if (maxRadiance > 0.0f) c = {std::fmin(c.x, maxRadiance), std::fmin(c.y, maxRadiance), std::fmin(c.z, maxRadiance)};
            float wgt = std::fmax(lum(c), 0.0f) * solid;
            weights[(size_t)y * w + x] = wgt;
            total += wgt;
        }
    }
    if (!(total > 0.0f)) return 0;
    float cumulative = 0.0f;
    for (size_t i = 0; i < weights.size(); ++i) {
        cumulative += weights[i];
        uint32_t y = (uint32_t)(i / w);
        float theta = ((float)y + 0.5f) * dTheta;
        float solid = std::fmax(std::sin(theta) * dTheta * dPhi, 1e-8f);
        float prob = weights[i] / total;
        out[i].cdf = std::fmin(cumulative / total, 1.0f);
        out[i].pdf_solid_angle = prob / solid;
    }
    return (uint32_t)weights.size();
}

}  // extern "C"
