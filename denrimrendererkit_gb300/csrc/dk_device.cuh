// Device-side scene model, BVH traversal and shading of the sm_103a wavefront
// path tracer.  Each function restates the named function of the reference
// shader (Sources/DenrimRendererKit/Resources/Shaders/PathTrace.metal); the
// kernels in dk_kernels.cu split the reference's per-pixel loop
// (pathTraceKernel, PathTrace.metal:5167-5586) into extend / shade / shadow
// stages over SoA path queues.
#pragma once
#include <cstdint>

#include "../../include/denrim_cuda.h"
#include "dk_kernels.h"
#include "dk_math.cuh"

namespace dk {

// ------------------------------------------------------------- scene ------
// Leaf children are encoded as 0x80000000 | first << 3 | (count - 1).
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kStackSize = 64;
constexpr uint32_t kNoHit = 0xffffffffu;

struct Ray { float3 origin, direction; };

// Hit (PathTrace.metal:229-253) for triangle hits.
struct Hit {
    float t;
    float3 position;
    float3 normal;
    float2 uv;
    float3 tangent;
    float3 bitangent;
    uint32_t materialID;
    uint32_t materialID2;
    float materialBlend;
    uint32_t objectID;
    uint32_t primitiveID;
    bool frontFacing;
};

struct HitRec { float t; uint32_t tri; float u, v; };

// ------------------------------------------------------- traversal --------
// intersectBounds (PathTrace.metal:1854-1863) on one child box, exact ops.
__device__ __forceinline__ bool childBox(float bx0, float bx1, float by0, float by1, float bz0, float bz1,
                                         float3 o, float3 inv, float closestT, float& tNear) {
    float tx0 = ex::mul(ex::sub(bx0, o.x), inv.x), tx1 = ex::mul(ex::sub(bx1, o.x), inv.x);
    float ty0 = ex::mul(ex::sub(by0, o.y), inv.y), ty1 = ex::mul(ex::sub(by1, o.y), inv.y);
    float tz0 = ex::mul(ex::sub(bz0, o.z), inv.z), tz1 = ex::mul(ex::sub(bz1, o.z), inv.z);
    float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), 0.0f));
    float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), closestT));
    tNear = tn;
    return tn <= tf;
}

// The slab test of the watertight mode (after Ize, "Robust BVH Ray
// Traversal", JCGT 2(2), 2013): a ray that lies in a slab's boundary plane
// (0 x inf = NaN) counts as inside the slab, and the far distance is widened
// by 1 + 2 gamma(3) so that rounding never culls a box the ray touches.  The
// reference's test above drops such boxes, so a ray along a grid plane of a
// tessellated surface can miss every triangle around it whatever the
// triangle test.
__device__ __forceinline__ float nanTo(float x, float v) { return x != x ? v : x; }

__device__ __forceinline__ bool childBoxRobust(float bx0, float bx1, float by0, float by1, float bz0, float bz1,
                                               float3 o, float3 inv, float closestT, float& tNear) {
    const float tx0 = ex::mul(ex::sub(bx0, o.x), inv.x), tx1 = ex::mul(ex::sub(bx1, o.x), inv.x);
    const float ty0 = ex::mul(ex::sub(by0, o.y), inv.y), ty1 = ex::mul(ex::sub(by1, o.y), inv.y);
    const float tz0 = ex::mul(ex::sub(bz0, o.z), inv.z), tz1 = ex::mul(ex::sub(bz1, o.z), inv.z);
    const float nx = fminf(nanTo(tx0, -INFINITY), nanTo(tx1, -INFINITY));
    const float fx = fmaxf(nanTo(tx0, INFINITY), nanTo(tx1, INFINITY));
    const float ny = fminf(nanTo(ty0, -INFINITY), nanTo(ty1, -INFINITY));
    const float fy = fmaxf(nanTo(ty0, INFINITY), nanTo(ty1, INFINITY));
    const float nz = fminf(nanTo(tz0, -INFINITY), nanTo(tz1, -INFINITY));
    const float fz = fmaxf(nanTo(tz0, INFINITY), nanTo(tz1, INFINITY));
    const float tn = fmaxf(fmaxf(nx, ny), fmaxf(nz, 0.0f));
    const float tf = fminf(ex::mul(fminf(fminf(fx, fy), fz), 1.0000004f), closestT);
    tNear = tn;
    return tn <= tf;
}

// Möller-Trumbore as intersectTriangle (PathTrace.metal:1801-1852), exact ops.
__device__ __forceinline__ bool mtTest(float3 o, float3 d, float3 v0, float3 e1, float3 e2, float& t, float& u,
                                       float& v) {
    float3 p = ex::cross(d, e2);
    float det = ex::dot(e1, p);
    if (fabsf(det) < 1e-7f) return false;
    float inv = ex::rcp(det);
    float3 s = ex::sub(o, v0);
    u = ex::mul(inv, ex::dot(s, p));
    if (u < 0.0f || u > 1.0f) return false;
    float3 q = ex::cross(s, e1);
    v = ex::mul(inv, ex::dot(d, q));
    if (v < 0.0f || ex::add(u, v) > 1.0f) return false;
    t = ex::mul(inv, ex::dot(e2, q));
    return t > 0.0005f;
}

// Watertight ray-triangle test (Woop, Benthin and Wald, "Watertight
// Ray/Triangle Intersection", JCGT 2(1), 2013), the option beside the
// reference's Moller-Trumbore: the ray is sheared so that it runs along +z
// through the origin, and the 2-D edge functions of the sheared vertices
// decide the hit.  A shared edge gives the same function (with opposite sign)
// to both of its triangles -- every product and difference is rounded on its
// own, never contracted -- so a ray through an edge or a vertex cannot slip
// between neighbours; an edge function that rounds to zero is recomputed in
// FP64.  Same outputs as mtTest: t (> 0.0005, the reference's self-hit
// offset), u = weight of v1, v = weight of v2.
__device__ __forceinline__ float axisOf(float3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }

__device__ __forceinline__ bool wtTest(float3 o, float3 d, float3 v0, float3 v1, float3 v2, float& t, float& u,
                                       float& v) {
    const float adx = fabsf(d.x), ady = fabsf(d.y), adz = fabsf(d.z);
    const int kz = adx > ady ? (adx > adz ? 0 : 2) : (ady > adz ? 1 : 2);
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    const float dz = axisOf(d, kz);
    if (dz < 0.0f) {  // keep the winding of the sheared triangle
        const int k = kx;
        kx = ky;
        ky = k;
    }
    const float sx = ex::div(axisOf(d, kx), dz), sy = ex::div(axisOf(d, ky), dz), sz = ex::rcp(dz);
    const float3 A = ex::sub(v0, o), B = ex::sub(v1, o), C = ex::sub(v2, o);
    const float az = axisOf(A, kz), bz = axisOf(B, kz), cz = axisOf(C, kz);
    const float ax = ex::sub(axisOf(A, kx), ex::mul(sx, az)), ay = ex::sub(axisOf(A, ky), ex::mul(sy, az));
    const float bx = ex::sub(axisOf(B, kx), ex::mul(sx, bz)), by = ex::sub(axisOf(B, ky), ex::mul(sy, bz));
    const float cx = ex::sub(axisOf(C, kx), ex::mul(sx, cz)), cy = ex::sub(axisOf(C, ky), ex::mul(sy, cz));
    float U = ex::sub(ex::mul(cx, by), ex::mul(cy, bx));
    float V = ex::sub(ex::mul(ax, cy), ex::mul(ay, cx));
    float W = ex::sub(ex::mul(bx, ay), ex::mul(by, ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)__dsub_rn(__dmul_rn((double)cx, (double)by), __dmul_rn((double)cy, (double)bx));
        V = (float)__dsub_rn(__dmul_rn((double)ax, (double)cy), __dmul_rn((double)ay, (double)cx));
        W = (float)__dsub_rn(__dmul_rn((double)bx, (double)ay), __dmul_rn((double)by, (double)ax));
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    const float det = ex::add(ex::add(U, V), W);
    if (det == 0.0f) return false;
    const float T = ex::add(ex::add(ex::mul(U, ex::mul(sz, az)), ex::mul(V, ex::mul(sz, bz))), ex::mul(W, ex::mul(sz, cz)));
    const float inv = ex::rcp(det);
    t = ex::mul(T, inv);
    u = ex::mul(V, inv);
    v = ex::mul(W, inv);
    return t > 0.0005f;
}

// The scene's triangle test on one slot's rows (v0, slot), (e1 | v1, triangle),
// (e2 | v2, flags): Moller-Trumbore over edges (the reference's test, the
// default) or the watertight test over absolute vertices.
__device__ __forceinline__ bool triTest(const DevScene& S, float3 o, float3 d, const float4& a, const float4& b,
                                        const float4& c, float& t, float& u, float& v) {
    if (S.watertight) return wtTest(o, d, xyz(a), xyz(b), xyz(c), t, u, v);
    return mtTest(o, d, xyz(a), xyz(b), xyz(c), t, u, v);
}

__device__ __forceinline__ float3 rcp3(float3 d) { return f3(ex::rcp(d.x), ex::rcp(d.y), ex::rcp(d.z)); }

// The children of a 4-wide node (8 x float4: x/y/z slab rows with one lane per
// child, then the child references) whose boxes the ray enters no later than
// `tmax`, nearest first.  Misses sort behind the hits with t = +inf.
struct Wide {
    uint32_t c0, c1, c2, c3;
    float t0, t1, t2, t3;
};

__device__ __forceinline__ void wideSwap(uint32_t& ca, float& ta, uint32_t& cb, float& tb) {
    if (tb < ta) {
        float t = ta;
        ta = tb;
        tb = t;
        uint32_t c = ca;
        ca = cb;
        cb = c;
    }
}

template <bool kSort = true>
__device__ __forceinline__ int wideVisit(const DevScene& S, uint32_t node, float3 o, float3 inv, float tmax, Wide& w) {
    const float4* n = S.nodes + 8 * (size_t)node;
    float4 lx = __ldg(n + 0), hx = __ldg(n + 1), ly = __ldg(n + 2), hy = __ldg(n + 3), lz = __ldg(n + 4),
           hz = __ldg(n + 5);
    uint4 ch = __ldg(reinterpret_cast<const uint4*>(n + 6));
    float t;
    w.c0 = ch.x;
    w.c1 = ch.y;
    w.c2 = ch.z;
    w.c3 = ch.w;
    if (S.watertight) {
        w.t0 = childBoxRobust(lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, o, inv, tmax, t) ? t : INFINITY;
        w.t1 = childBoxRobust(lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, o, inv, tmax, t) ? t : INFINITY;
        w.t2 = childBoxRobust(lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, o, inv, tmax, t) ? t : INFINITY;
        w.t3 = childBoxRobust(lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, o, inv, tmax, t) ? t : INFINITY;
    } else {
        w.t0 = childBox(lx.x, hx.x, ly.x, hy.x, lz.x, hz.x, o, inv, tmax, t) ? t : INFINITY;
        w.t1 = childBox(lx.y, hx.y, ly.y, hy.y, lz.y, hz.y, o, inv, tmax, t) ? t : INFINITY;
        w.t2 = childBox(lx.z, hx.z, ly.z, hy.z, lz.z, hz.z, o, inv, tmax, t) ? t : INFINITY;
        w.t3 = childBox(lx.w, hx.w, ly.w, hy.w, lz.w, hz.w, o, inv, tmax, t) ? t : INFINITY;
    }
    int k = (w.t0 != INFINITY) + (w.t1 != INFINITY) + (w.t2 != INFINITY) + (w.t3 != INFINITY);
    if (!kSort) return k;  // lanes in child order, misses at t = +inf
    if (k > 1) {
        wideSwap(w.c0, w.t0, w.c1, w.t1);
        wideSwap(w.c2, w.t2, w.c3, w.t3);
        wideSwap(w.c0, w.t0, w.c2, w.t2);
        wideSwap(w.c1, w.t1, w.c3, w.t3);
        wideSwap(w.c1, w.t1, w.c2, w.t2);
    } else if (k == 1) {  // move the single hit to lane 0
        if (w.t1 != INFINITY) { w.c0 = w.c1; w.t0 = w.t1; }
        if (w.t2 != INFINITY) { w.c0 = w.c2; w.t0 = w.t2; }
        if (w.t3 != INFINITY) { w.c0 = w.c3; w.t0 = w.t3; }
    }
    return k;
}

// Closest hit.  Returns argmin over (t, reference leaf slot): the reference's
// strict `t < closest.t` under left-first DFS picks, among equal t, the
// triangle that comes first in its primitiveIndices order, which is the slot.
__device__ HitRec traceClosest(const DevScene& S, float3 o, float3 d) {
    HitRec best;
    best.t = INFINITY;
    best.tri = kNoHit;
    best.u = 0.0f;
    best.v = 0.0f;
    uint32_t bestSlot = 0xffffffffu;
    if (S.node_count == 0) return best;
    float3 inv = rcp3(d);
    int stackNode[kStackSize];
    float stackT[kStackSize];
    int sp = 0;
    uint32_t node = 0;
    for (;;) {
        if ((node & kLeafBit) == 0) {
            Wide w;
            int k = wideVisit(S, node, o, inv, best.t, w);
            if (k > 0) {
                if (k > 3) { stackNode[sp] = (int)w.c3; stackT[sp] = w.t3; ++sp; }
                if (k > 2) { stackNode[sp] = (int)w.c2; stackT[sp] = w.t2; ++sp; }
                if (k > 1) { stackNode[sp] = (int)w.c1; stackT[sp] = w.t1; ++sp; }
                node = w.c0;
                continue;
            }
        } else {
            uint32_t first = (node & ~kLeafBit) >> 3;
            uint32_t cnt = (node & 7u) + 1u;
            for (uint32_t i = first; i < first + cnt; ++i) {
                const float4* q = S.isect + 3 * (size_t)i;
                float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2);
                float t, u, v;
                if (triTest(S, o, d, a, b, c, t, u, v)) {
                    uint32_t slot = __float_as_uint(a.w);
                    if (t < best.t || (t == best.t && slot < bestSlot)) {
                        best.t = t;
                        best.u = u;
                        best.v = v;
                        best.tri = __float_as_uint(b.w);
                        bestSlot = slot;
                    }
                }
            }
        }
        bool found = false;
        while (sp > 0) {
            --sp;
            if (stackT[sp] <= best.t) {
                node = (uint32_t)stackNode[sp];
                found = true;
                break;
            }
        }
        if (!found) break;
    }
    return best;
}

// ---------------------------------------------- resumable traversal ------
// The persistent kernels advance each lane's ray a bounded number of node or
// leaf visits at a time and refill finished lanes with new rays, so a warp's
// lanes stay busy instead of waiting for the warp's longest traversal.
struct ClosestState {
    float3 o, d, inv;
    float bestT, bu, bv;
    uint32_t bestTri, bestSlot, node;
    int sp;
};

__device__ __forceinline__ void closestInit(ClosestState& st, float3 o, float3 d) {
    st.o = o;
    st.d = d;
    st.inv = rcp3(d);
    st.bestT = INFINITY;
    st.bu = st.bv = 0.0f;
    st.bestTri = kNoHit;
    st.bestSlot = 0xffffffffu;
    st.node = 0;
    st.sp = 0;
}

// Up to `budget` visits of the closest-hit traversal of traceClosest; returns
// true when the ray is finished.
__device__ __forceinline__ bool closestSteps(const DevScene& S, ClosestState& st, int* stackNode, float* stackT,
                                             int budget) {
    for (int it = 0; it < budget; ++it) {
        if ((st.node & kLeafBit) == 0) {
            Wide w;
            int k = wideVisit(S, st.node, st.o, st.inv, st.bestT, w);
            if (k > 0) {
                if (k > 3) { stackNode[st.sp] = (int)w.c3; stackT[st.sp] = w.t3; ++st.sp; }
                if (k > 2) { stackNode[st.sp] = (int)w.c2; stackT[st.sp] = w.t2; ++st.sp; }
                if (k > 1) { stackNode[st.sp] = (int)w.c1; stackT[st.sp] = w.t1; ++st.sp; }
                st.node = w.c0;
                continue;
            }
        } else {
            uint32_t first = (st.node & ~kLeafBit) >> 3;
            uint32_t cnt = (st.node & 7u) + 1u;
            for (uint32_t i = first; i < first + cnt; ++i) {
                const float4* q = S.isect + 3 * (size_t)i;
                float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2);
                float t, u, v;
                if (triTest(S, st.o, st.d, a, b, c, t, u, v)) {
                    uint32_t slot = __float_as_uint(a.w);
                    if (t < st.bestT || (t == st.bestT && slot < st.bestSlot)) {
                        st.bestT = t;
                        st.bu = u;
                        st.bv = v;
                        st.bestTri = __float_as_uint(b.w);
                        st.bestSlot = slot;
                    }
                }
            }
        }
        bool found = false;
        while (st.sp > 0) {
            --st.sp;
            if (stackT[st.sp] <= st.bestT) {
                st.node = (uint32_t)stackNode[st.sp];
                found = true;
                break;
            }
        }
        if (!found) return true;
    }
    return false;
}

// Whether a triangle slot's flags block a shadow ray for a render whose
// material table has opacity bits `mask` (material IDs below 32).
__device__ __forceinline__ bool blocksShadow(uint32_t flags, uint32_t mask) {
    uint32_t mid = flags >> 8;
    return mid < 32u ? ((mask >> mid) & 1u) != 0u : (flags & 1u) != 0u;
}

// `rec` (may be null) receives the first kRecLayers non-opaque triangles the
// query crosses as (t bits, slot); `recCount` counts them, `recOverflow` marks
// more.
struct AnyState {
    float3 o, d, inv;
    float tmax;
    uint32_t node;
    uint32_t opaqueMask;
    int sp;
    bool sawNonOpaque;
    bool recOverflow;
    uint32_t recCount;
    uint2* rec;
};

__device__ __forceinline__ void anyInit(AnyState& st, float3 o, float3 d, float tmax, uint32_t opaqueMask,
                                        uint2* rec) {
    st.o = o;
    st.d = d;
    st.inv = rcp3(d);
    st.tmax = tmax;
    st.node = 0;
    st.opaqueMask = opaqueMask;
    st.sp = 0;
    st.sawNonOpaque = false;
    st.recOverflow = false;
    st.recCount = 0;
    st.rec = rec;
}

// Children of an any-hit query are visited in the SAH tree's left-right order
// (DK_ANY_SORTED=0, the default) or nearest first (1): an any-hit query needs
// no order for its answer, and skipping the sort is the faster of the two.
#ifndef DK_ANY_SORTED
#define DK_ANY_SORTED 0
#endif
// Up to `budget` node visits of the any-hit query over shadow-blocking
// triangles with 0.0005 < t < tmax: 0 running, 1 finished without an
// opaque blocker, 2 occluded.
__device__ __forceinline__ int anySteps(const DevScene& S, AnyState& st, int* stackNode, int budget) {
    for (int it = 0; it < budget; ++it) {
        if ((st.node & kLeafBit) == 0) {
            Wide w;
            int k = wideVisit<DK_ANY_SORTED != 0>(S, st.node, st.o, st.inv, st.tmax, w);
            if (k > 0 && !DK_ANY_SORTED) {  // first hit child next, the others pushed
                const uint32_t cA = w.c0, cB = w.c1, cC = w.c2, cD = w.c3;
                const bool hA = w.t0 != INFINITY, hB = w.t1 != INFINITY, hC = w.t2 != INFINITY, hD = w.t3 != INFINITY;
                uint32_t next = 0u;
                bool have = false;
                if (hD) { next = cD; have = true; }
                if (hC) { if (have) stackNode[st.sp++] = (int)next; next = cC; have = true; }
                if (hB) { if (have) stackNode[st.sp++] = (int)next; next = cB; have = true; }
                if (hA) { if (have) stackNode[st.sp++] = (int)next; next = cA; }
                st.node = next;
                continue;
            }
            if (k > 0) {
                if (k > 3) stackNode[st.sp++] = (int)w.c3;
                if (k > 2) stackNode[st.sp++] = (int)w.c2;
                if (k > 1) stackNode[st.sp++] = (int)w.c1;
                st.node = w.c0;
                continue;
            }
        } else {
            uint32_t first = (st.node & ~kLeafBit) >> 3;
            uint32_t cnt = (st.node & 7u) + 1u;
            for (uint32_t i = first; i < first + cnt; ++i) {
                const float4* q = S.isect + 3 * (size_t)i;
                float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2);
                float t, u, v;
                if (triTest(S, st.o, st.d, a, b, c, t, u, v) && t < st.tmax) {
                    if (blocksShadow(__float_as_uint(c.w), st.opaqueMask)) return 2;
                    st.sawNonOpaque = true;
                    if (st.rec) {
                        if (st.recCount < kRecLayers)
                            st.rec[st.recCount++] = make_uint2(__float_as_uint(t), i);
                        else
                            st.recOverflow = true;
                    }
                }
            }
        }
        if (st.sp == 0) return 1;
        st.node = (uint32_t)stackNode[--st.sp];
    }
    return 0;
}

// ------------------------------------- 8-wide quantised traversal ------
// The alternative layout (DevScene::wide8; node layout in dk_bvh.cu): child
// boxes quantised to 8 bits per bound against a per-node origin and
// power-of-two steps, rounded outwards, so a box test never rejects a child
// whose exact box the ray enters.  The traversal state holds two groups:
// interior children still to visit (first child index; interior mask << 8 |
// visit mask, bit slot ^ oct) and leaf slots still to test (first slot;
// 32-bit mask).  The builder puts the child lying furthest towards box corner
// c in slot c, so a ray whose direction signs form oct meets slot oct first
// and visiting by increasing slot ^ oct is roughly front to back.  A node
// visit pushes at most one group, so the stack depth is bounded by the tree
// depth (checked when the tree is built).
struct Trav {
    float3 o, d, inv;
    uint32_t oct;   // sign bits of the direction: x, y, z
    uint2 group;
    uint2 tris;
    int sp;
};

// Reciprocal direction for the box tests: a zero component is taken as
// +-1e-20 so that every slab distance stays finite.
__device__ __forceinline__ float3 boxInv(float3 d) {
    auto r = [](float v) { return 1.0f / (fabsf(v) < 1e-20f ? copysignf(1e-20f, v) : v); };
    return f3(r(d.x), r(d.y), r(d.z));
}

__device__ __forceinline__ void travInit(Trav& t, float3 o, float3 d) {
    t.o = o;
    t.d = d;
    t.inv = boxInv(d);
    t.oct = (t.inv.x < 0.0f ? 1u : 0u) | (t.inv.y < 0.0f ? 2u : 0u) | (t.inv.z < 0.0f ? 4u : 0u);
    t.group = make_uint2(0u, (1u << 8) | (1u << t.oct));  // the root: slot 0 of a one-child group
    t.tris = make_uint2(0u, 0u);
    t.sp = 0;
}

// Byte j of `w` as a float: 2^23 + b assembled by a byte permute, minus 2^23.
__device__ __forceinline__ float qByte(uint32_t w, uint32_t j) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | j)) - 8388608.0f;
}

// Tests the eight child boxes of `node` against (0, tmax]; the hit interior
// children become the current group, the hit leaves' slots the triangle set.
__device__ __forceinline__ void visit8(const DevScene& S, Trav& t, uint32_t node, float tmax) {
    const uint4* n = reinterpret_cast<const uint4*>(S.nodes) + 5 * (size_t)node;
    const uint4 w0 = __ldg(n + 0), w1 = __ldg(n + 1), w2 = __ldg(n + 2), w3 = __ldg(n + 3), w4 = __ldg(n + 4);
    const float ax = __uint_as_float((w0.w & 0xffu) << 23) * t.inv.x;
    const float ay = __uint_as_float(((w0.w >> 8) & 0xffu) << 23) * t.inv.y;
    const float az = __uint_as_float(((w0.w >> 16) & 0xffu) << 23) * t.inv.z;
    const float bx = (__uint_as_float(w0.x) - t.o.x) * t.inv.x;
    const float by = (__uint_as_float(w0.y) - t.o.y) * t.inv.y;
    const float bz = (__uint_as_float(w0.z) - t.o.z) * t.inv.z;
    const uint32_t imask = w0.w >> 24;
    // Near and far planes per axis by the sign of the direction.
    const bool sx = t.oct & 1u, sy = t.oct & 2u, sz = t.oct & 4u;
    const uint32_t nx[2] = {sx ? w3.z : w2.x, sx ? w3.w : w2.y}, fx[2] = {sx ? w2.x : w3.z, sx ? w2.y : w3.w};
    const uint32_t ny[2] = {sy ? w4.x : w2.z, sy ? w4.y : w2.w}, fy[2] = {sy ? w2.z : w4.x, sy ? w2.w : w4.y};
    const uint32_t nz[2] = {sz ? w4.z : w3.x, sz ? w4.w : w3.y}, fz[2] = {sz ? w3.x : w4.z, sz ? w3.y : w4.w};
    const uint32_t meta[2] = {w1.z, w1.w};
    uint32_t order = 0u, triMask = 0u;
#pragma unroll
    for (uint32_t h = 0; h < 2; ++h) {
#pragma unroll
        for (uint32_t j = 0; j < 4; ++j) {
            const uint32_t s = 4u * h + j;
            float tn = fmaxf(fmaxf(fmaf(qByte(nx[h], j), ax, bx), fmaf(qByte(ny[h], j), ay, by)),
                             fmaxf(fmaf(qByte(nz[h], j), az, bz), 0.0f));
            float tf = fminf(fminf(fmaf(qByte(fx[h], j), ax, bx), fmaf(qByte(fy[h], j), ay, by)),
                             fminf(fmaf(qByte(fz[h], j), az, bz), tmax));
            if (tn <= tf) {
                const uint32_t m = (meta[h] >> (8u * j)) & 0xffu;
                triMask |= ((1u << (m >> 5)) - 1u) << (m & 31u);
                order |= ((imask >> s) & 1u) << (s ^ t.oct);
            }
        }
    }
    t.group = make_uint2(w1.x, (imask << 8) | order);
    t.tris = make_uint2(w1.y, triMask);
}

// Up to `budget` node visits, each followed by the triangles of the leaves
// it hit; `leaf(slot, tmax)` tests one leaf slot (it may lower tmax) and
// returns true to stop the query.  Returns 0 running, 1 finished, 2 stopped.
template <class LeafFn>
__device__ __forceinline__ int travSteps(const DevScene& S, Trav& t, uint2* stack, float& tmax, int budget,
                                         LeafFn&& leaf) {
    for (int it = 0;; ++it) {
        while (t.tris.y) {
            const uint32_t j = __ffs(t.tris.y) - 1;
            t.tris.y &= t.tris.y - 1u;
            if (leaf(t.tris.x + j, tmax)) return 2;
        }
        if ((t.group.y & 0xffu) == 0u) {
            if (t.sp == 0) return 1;
            t.group = stack[--t.sp];
        }
        if (it == budget) return 0;
        const uint32_t k = __ffs(t.group.y & 0xffu) - 1;
        t.group.y &= ~(1u << k);
        const uint32_t s = k ^ t.oct;
        const uint32_t node = t.group.x + __popc((t.group.y >> 8) & ((1u << s) - 1u));
        if (t.group.y & 0xffu) stack[t.sp++] = t.group;
        visit8(S, t, node, tmax);
    }
}

// Closest hit over the 8-wide tree, the same (t, slot) argmin as above.
struct Closest8 {
    Trav tr;
    float bestT, bu, bv;
    uint32_t bestTri, bestSlot;
};

__device__ __forceinline__ void closestInit(Closest8& st, float3 o, float3 d) {
    travInit(st.tr, o, d);
    st.bestT = INFINITY;
    st.bu = st.bv = 0.0f;
    st.bestTri = kNoHit;
    st.bestSlot = 0xffffffffu;
}

__device__ __forceinline__ bool closestSteps(const DevScene& S, Closest8& st, uint2* stack, int budget) {
    if (S.node_count == 0) return true;
    const float3 o = st.tr.o, d = st.tr.d;
    return travSteps(S, st.tr, stack, st.bestT, budget, [&](uint32_t i, float& tmax) {
        const float4* q = S.isect + 3 * (size_t)i;
        const float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2);
        float t, u, v;
        if (triTest(S, o, d, a, b, c, t, u, v)) {
            const uint32_t slot = __float_as_uint(a.w);
            if (t < tmax || (t == tmax && slot < st.bestSlot)) {
                tmax = t;
                st.bu = u;
                st.bv = v;
                st.bestTri = __float_as_uint(b.w);
                st.bestSlot = slot;
            }
        }
        return false;
    }) != 0;
}

__device__ __noinline__ HitRec traceClosest8(const DevScene& S, float3 o, float3 d) {
    Closest8 st;
    uint2 stack[kTraversalStack];
    closestInit(st, o, d);
    closestSteps(S, st, stack, 1 << 30);
    return HitRec{st.bestT, st.bestTri, st.bu, st.bv};
}

// Any hit over the 8-wide tree (the AnyState query above).
struct Any8 {
    Trav tr;
    float tmax;
    uint32_t opaqueMask;
    bool sawNonOpaque;
    bool recOverflow;
    uint32_t recCount;
    uint2* rec;
};

__device__ __forceinline__ void anyInit(Any8& st, float3 o, float3 d, float tmax, uint32_t opaqueMask, uint2* rec) {
    travInit(st.tr, o, d);
    st.tmax = tmax;
    st.opaqueMask = opaqueMask;
    st.sawNonOpaque = false;
    st.recOverflow = false;
    st.recCount = 0;
    st.rec = rec;
}

__device__ __forceinline__ int anySteps(const DevScene& S, Any8& st, uint2* stack, int budget) {
    if (S.node_count == 0) return 1;
    const float3 o = st.tr.o, d = st.tr.d;
    float tmax = st.tmax;
    return travSteps(S, st.tr, stack, tmax, budget, [&](uint32_t i, float&) {
        const float4* q = S.isect + 3 * (size_t)i;
        const float4 a = __ldg(q + 0), b = __ldg(q + 1), c = __ldg(q + 2);
        float t, u, v;
        if (triTest(S, o, d, a, b, c, t, u, v) && t < st.tmax) {
            if (blocksShadow(__float_as_uint(c.w), st.opaqueMask)) return true;
            st.sawNonOpaque = true;
            if (st.rec) {
                if (st.recCount < kRecLayers)
                    st.rec[st.recCount++] = make_uint2(__float_as_uint(t), i);
                else
                    st.recOverflow = true;
            }
        }
        return false;
    });
}

// Hit attributes of intersectTriangle / intersectScene (PathTrace.metal:
// 1840-1851, 3366-3380) from the traversal's (t, u, v), exact ops.
__device__ __forceinline__ Hit makeHit(const DevScene& S, const Ray& ray, const HitRec& r) {
    const dk_triangle& tri = S.tris[r.tri];
    Hit h;
    h.t = r.t;
    h.position = ex::add(ray.origin, ex::mul(r.t, ray.direction));
    float w = ex::sub(ex::sub(1.0f, r.u), r.v);
    float4 n0 = __ldg(reinterpret_cast<const float4*>(&tri.n0));
    float4 n1 = __ldg(reinterpret_cast<const float4*>(&tri.n1));
    float4 n2 = __ldg(reinterpret_cast<const float4*>(&tri.n2));
    float3 nn = ex::add(ex::add(ex::mul(w, xyz(n0)), ex::mul(r.u, xyz(n1))), ex::mul(r.v, xyz(n2)));
    float3 normal = ex::normalize(nn);
    float nd = ex::dot(normal, ray.direction);
    h.frontFacing = nd <= 0.0f;
    if (nd > 0.0f) normal = -normal;
    h.normal = normal;
    float4 t0 = __ldg(reinterpret_cast<const float4*>(&tri.uv0));
    float4 t1 = __ldg(reinterpret_cast<const float4*>(&tri.uv1));
    float4 t2 = __ldg(reinterpret_cast<const float4*>(&tri.uv2));
    h.uv = make_float2(ex::add(ex::add(ex::mul(w, t0.x), ex::mul(r.u, t1.x)), ex::mul(r.v, t2.x)),
                       ex::add(ex::add(ex::mul(w, t0.y), ex::mul(r.u, t1.y)), ex::mul(r.v, t2.y)));
    h.tangent = ex::normalize(xyz(__ldg(reinterpret_cast<const float4*>(&tri.tangent))));
    h.bitangent = ex::normalize(xyz(__ldg(reinterpret_cast<const float4*>(&tri.bitangent))));
    uint4 ids = __ldg(reinterpret_cast<const uint4*>(&tri.material_id));
    h.materialID = ids.x;
    h.materialID2 = ids.x;
    h.materialBlend = 0.0f;
    h.objectID = ids.y;
    h.primitiveID = r.tri;
    return h;
}

}  // namespace dk
