// Host side of the C ABI declared in include/denrim_cuda.h: device and
// session management, the scene upload with the traversal-BVH conversion, the
// per-sample batch scheduler, readback, and the scene-compile helpers that
// restate the reference's Swift host builders.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <future>
#include <mutex>
#include <cstring>
#include <string>
#include <thread>

#include <cuda_fp16.h>
#include <vector>

#include "dk_host.h"

namespace dk {

namespace {
thread_local std::string g_error;
int g_device = -1;
cudaDeviceProp g_prop;
}  // namespace

int fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}

// Lets other translation units of the library report through dk_last_error_message().
void setLastError(const std::string& message) { g_error = message; }

int ensureDevice() {
    if (g_device >= 0) return DK_OK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(DK_ERROR_NO_DEVICE, "No compatible CUDA device is available.");
    }
    if (cudaSetDevice(0) != cudaSuccess) return fail(DK_ERROR_NO_DEVICE, "cudaSetDevice(0) failed.");
    cudaGetDeviceProperties(&g_prop, 0);
    g_device = 0;
    return DK_OK;
}

const cudaDeviceProp& deviceProp() { return g_prop; }

int openDevice(int ordinal) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(DK_ERROR_NO_DEVICE, "No compatible CUDA device is available.");
    }
    if (ordinal < 0 || ordinal >= n) return fail(DK_ERROR_INVALID_ARGUMENT, "device ordinal out of range");
    DK_CUDA(cudaSetDevice(ordinal), "cudaSetDevice");
    DK_CUDA(cudaGetDeviceProperties(&g_prop, ordinal), "cudaGetDeviceProperties");
    if (g_prop.major < 10) return fail(DK_ERROR_MISSING_KERNEL, "this library carries sm_103a kernels only");
    g_device = ordinal;
    return DK_OK;
}

const char* lastError() { return g_error.c_str(); }

}  // namespace dk

namespace {

using dk::fail;

// ------------------------------------------------------ BVH builder -------
// BVHBuilder.build (Acceleration/BVHBuilder.swift:7-135) + BVHFlattener
// (FlatBVH.swift:13-32).  The median split makes every subtree's node count a
// function of its primitive count alone, so pre-order node indices are known
// before the subtrees are built and the top levels can be built in parallel.
struct BBox {
    float mn[3], mx[3];
};
inline BBox emptyBox() { return {{FLT_MAX, FLT_MAX, FLT_MAX}, {-FLT_MAX, -FLT_MAX, -FLT_MAX}}; }
inline void grow(BBox& b, const float* p) {
    for (int a = 0; a < 3; ++a) {
        b.mn[a] = std::fmin(b.mn[a], p[a]);
        b.mx[a] = std::fmax(b.mx[a], p[a]);
    }
}

struct BvhBuild {
    const std::vector<BBox>* prim;
    std::vector<float> centroid;  // 3 per primitive
    uint32_t* idx;
    dk_bvh_node* out;
    uint32_t maxLeaf;

    uint64_t subtreeNodes(uint64_t n) const {
        if (n <= std::max<uint64_t>(1, maxLeaf)) return 1;
        return 1 + subtreeNodes(n / 2) + subtreeNodes(n - n / 2);
    }

    void build(uint32_t lo, uint32_t hi, uint32_t nodeIndex, int depth) {
        BBox b = emptyBox();
        for (uint32_t i = lo; i < hi; ++i) {
            grow(b, (*prim)[idx[i]].mn);
            grow(b, (*prim)[idx[i]].mx);
        }
        uint32_t count = hi - lo;
        dk_bvh_node& n = out[nodeIndex];
        n.bounds_min = {b.mn[0], b.mn[1], b.mn[2], 0.0f};
        n.bounds_max = {b.mx[0], b.mx[1], b.mx[2], 0.0f};
        if (count <= std::max<uint32_t>(1, maxLeaf)) {
            n.metadata = {0u, 0u, lo, count};
            return;
        }
        BBox cb = emptyBox();
        for (uint32_t i = lo; i < hi; ++i) grow(cb, &centroid[3 * (size_t)idx[i]]);
        float e[3] = {cb.mx[0] - cb.mn[0], cb.mx[1] - cb.mn[1], cb.mx[2] - cb.mn[2]};
        int axis = (e[0] >= e[1] && e[0] >= e[2]) ? 0 : (e[1] >= e[2] ? 1 : 2);
        const float* c = centroid.data();
        std::stable_sort(idx + lo, idx + hi, [c, axis](uint32_t l, uint32_t r) {
            return c[3 * (size_t)l + axis] < c[3 * (size_t)r + axis];
        });
        uint32_t mid = lo + count / 2;
        uint32_t left = nodeIndex + 1;
        uint32_t right = left + (uint32_t)subtreeNodes(mid - lo);
        n.metadata = {left, right, 0u, 0u};
        if (depth < 4 && count > 65536) {
            std::thread t([=] { this->build(lo, mid, left, depth + 1); });
            build(mid, hi, right, depth + 1);
            t.join();
        } else {
            build(lo, mid, left, depth + 1);
            build(mid, hi, right, depth + 1);
        }
    }
};

uint32_t buildReferenceBvh(const dk_triangle* tris, uint32_t n, uint32_t maxLeaf, dk_bvh_node* nodes,
                           uint32_t* primIdx) {
    if (n == 0) return 0;
    std::vector<BBox> prim(n);
    BvhBuild b;
    b.centroid.resize(3 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
        BBox bb = emptyBox();
        grow(bb, &tris[i].v0.x);
        grow(bb, &tris[i].v1.x);
        grow(bb, &tris[i].v2.x);
        prim[i] = bb;
        for (int a = 0; a < 3; ++a) b.centroid[3 * (size_t)i + a] = (bb.mn[a] + bb.mx[a]) * 0.5f;
    }
    for (uint32_t i = 0; i < n; ++i) primIdx[i] = i;
    b.prim = &prim;
    b.idx = primIdx;
    b.out = nodes;
    b.maxLeaf = maxLeaf;
    uint32_t count = (uint32_t)b.subtreeNodes(n);
    b.build(0, n, 0, 0);
    return count;
}

// ----------------------------------------------------------- session ----
struct Session {
    dk_settings settings;
    dk::DevScene scene;
    dk::Wave wave;
    dk::Accum accum;
    dk::DevJob* jobs = nullptr;  // device copy of the wave's job table (one job)
    dk::Arena arena;
    float4* staging = nullptr;
    // One-wave renders replayed as CUDA graphs: the wave's kernel sequence for
    // a (tile, samples) key, captured on its first use.
    struct WaveGraph {
        uint32_t tx, ty, tw, th, nb, bounces;
        int aovs;
        cudaGraphExec_t exec;
        size_t events;
        std::vector<int> kinds;
        uint64_t launches;
    };
    std::vector<WaveGraph> graphs;
    bool graphsFailed = false;
    uint32_t* rgba8 = nullptr;     // display bytes (allocated on first use)
    uint32_t* encodeWs = nullptr;  // display-encoding workspace
    cudaEvent_t copyDone = nullptr;  // orders dk_session_copy_output before the caller's stream
    cudaStream_t stream = nullptr;
    std::vector<cudaEvent_t> evPool;
    uint32_t sampleCount = 0;
    dk_stats stats;
    dk::Grids grids;
    uint32_t opaqueMask = 0;
    unsigned long long* sdfCounters = nullptr;  // settings.collects_traversal_stats: the 13 SDF counters
};

void freeSession(Session* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (auto& g : s->graphs) cudaGraphExecDestroy(g.exec);
    s->arena.release();
    for (auto& e : s->evPool) cudaEventDestroy(e);
    if (s->copyDone) cudaEventDestroy(s->copyDone);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

}  // namespace

namespace dk {

int Arena::allocBytes(void** out, size_t n, const char* what) {
    *out = nullptr;
    if (n == 0) return DK_OK;
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, n);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return fail(e == cudaErrorMemoryAllocation ? DK_ERROR_OUT_OF_MEMORY : DK_ERROR_COMMAND_FAILED,
                    std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e));
    }
    buffers.push_back({p, n});
    bytes += n;
    *out = p;
    return DK_OK;
}

void Arena::release() {
    for (auto& b : buffers) cudaFree(b.ptr);
    buffers.clear();
    bytes = 0;
}

int kernelGrid(int which, int smCount);

Grids kernelGrids() {
    int sm = g_prop.multiProcessorCount;
    return Grids{kernelGrid(0, sm), kernelGrid(1, sm), kernelGrid(2, sm), kernelGrid(3, sm), kernelGrid(4, sm),
                 kernelGrid(5, sm), kernelGrid(6, sm), kernelGrid(7, sm)};
}

bool materialBlocksShadow(const dk_material& m) {
    float transmission = std::fmin(std::fmax(m.emission.w, 0.0f), 1.0f);
    return m.base_color.w > 0.001f && transmission <= 0.001f;
}

uint32_t opaqueMask(const dk_material* mats, uint32_t count) {
    uint32_t mask = 0;
    for (uint32_t i = 0; i < count && i < 32u; ++i)
        if (materialBlocksShadow(mats[i])) mask |= 1u << i;
    return mask;
}

int validateScene(const dk_scene* sc) {
    if (sc->triangle_count == 0 && sc->volume_count == 0)
        return fail(DK_ERROR_INVALID_SCENE, "Invalid render scene: Scene contains no renderable geometry.");
    if (sc->material_count == 0 || !sc->materials)
        return fail(DK_ERROR_INVALID_SCENE, "Invalid render scene: Scene contains no materials.");
    if (sc->volume_count != 0) {
        if (!sc->volumes) return fail(DK_ERROR_INVALID_ARGUMENT, "volumes is null while volume_count is not zero");
        for (uint32_t i = 0; i < sc->volume_count; ++i)
            if (sc->volumes[i].metadata.w != 1u)
                return fail(DK_ERROR_INVALID_SCENE,
                            "Invalid render scene: only sparse-brick distance volumes are supported by this backend.");
        if ((sc->volume_brick_count && !sc->volume_bricks) || (sc->volume_brick_sample_count && !sc->volume_brick_samples) ||
            (sc->volume_brick_grid_count && !sc->volume_brick_grids) ||
            (sc->volume_brick_grid_index_count && !sc->volume_brick_grid_indices))
            return fail(DK_ERROR_INVALID_ARGUMENT, "a volume array pointer is null while its count is not zero");
        if (sc->volume_brick_sample_count >= (1ull << 32) || sc->volume_brick_grid_index_count >= (1ull << 32))
            return fail(DK_ERROR_INVALID_SCENE, "Invalid render scene: volume arrays exceed 2^32 entries.");
    }
    if (sc->triangle_count && !sc->triangles) return fail(DK_ERROR_INVALID_ARGUMENT, "triangles is null");
    if ((sc->light_count && !sc->lights) || (sc->environment_sample_count && !sc->environment_samples) ||
        (sc->texture_descriptor_count && !sc->texture_descriptors) || (sc->texture_pixel_count && !sc->texture_pixels) ||
        (sc->node_count && !sc->nodes) || (sc->primitive_index_count && !sc->primitive_indices))
        return fail(DK_ERROR_INVALID_ARGUMENT, "a scene array pointer is null while its count is not zero");
    if (sc->environment_texture_index_plus_one > sc->texture_descriptor_count)
        return fail(DK_ERROR_INVALID_SCENE, "Invalid render scene: environment texture index out of range.");
    for (uint32_t i = 0; i < sc->texture_descriptor_count; ++i) {
        const dk_uint4& md = sc->texture_descriptors[i].metadata;
        if ((uint64_t)md.x + (uint64_t)md.y * md.z > sc->texture_pixel_count)
            return fail(DK_ERROR_INVALID_SCENE, "Invalid render scene: texture descriptor exceeds the pixel array.");
    }
    // Light records whose triangle is out of range are tolerated like the
    // reference: sampleDirectLighting skips them.
    return DK_OK;
}

// Traversal tree layout of the scenes uploaded from now on: DK_BVH_WIDTH=8
// selects the 8-wide quantised nodes, anything else the 4-wide FP32 nodes
// (the faster of the two on GB300, where the tree stays in L2 and traversal
// is bound by instruction issue).
static int traversalWidth() {
    const char* e = getenv("DK_BVH_WIDTH");
    return (e && e[0] == '8' && e[1] == 0) ? 8 : 4;
}

// DK_TRACE_CREATE=1: session-create phases (host wall time) on stderr.
bool traceCreate() {
    static const bool on = [] {
        const char* e = getenv("DK_TRACE_CREATE");
        return e && e[0] == '1';
    }();
    return on;
}

double wallMs() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// The traversal working set (triangle slots + nodes) as a persisting L2
// access-policy window of `stream`, opt-in (DK_L2_PERSIST=1): on the large
// scene it costs a fifth of the frame rate -- the 85 MB set-aside starves the
// shading stage's path-state and material traffic (k_shade 108 -> 162 ms)
// and the traversal stages gain nothing.  The set-aside is a limit of this
// process's context; the hit ratio scales the window to it.  Best effort: a
// refusal leaves the stream as it was.
void persistTraversal(const DevScene& D, cudaStream_t stream) {
    static const bool on = [] {
        const char* e = getenv("DK_L2_PERSIST");
        return e && e[0] == '1';
    }();
    if (!on || !D.isect || D.traversal_bytes == 0) return;
    int maxPersist = 0, maxWindow = 0;
    if (cudaDeviceGetAttribute(&maxPersist, cudaDevAttrMaxPersistingL2CacheSize, g_device) != cudaSuccess ||
        cudaDeviceGetAttribute(&maxWindow, cudaDevAttrMaxAccessPolicyWindowSize, g_device) != cudaSuccess ||
        maxPersist <= 0 || maxWindow <= 0) {
        cudaGetLastError();
        return;
    }
    static std::once_flag limitOnce;
    std::call_once(limitOnce, [&] {
        if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, (size_t)maxPersist) != cudaSuccess) cudaGetLastError();
    });
    size_t window = std::min<size_t>(D.traversal_bytes, (size_t)maxWindow);
    cudaStreamAttrValue v{};
    v.accessPolicyWindow.base_ptr = const_cast<float4*>(D.isect);
    v.accessPolicyWindow.num_bytes = window;
    v.accessPolicyWindow.hitRatio = std::min(1.0f, (float)maxPersist / (float)window);
    v.accessPolicyWindow.hitProp = cudaAccessPropertyPersisting;
    v.accessPolicyWindow.missProp = cudaAccessPropertyStreaming;
    if (cudaStreamSetAttribute(stream, cudaStreamAttributeAccessPolicyWindow, &v) != cudaSuccess) cudaGetLastError();
    if (traceCreate())
        fprintf(stderr, "[dk create] L2 window %.1f MB (set-aside %.1f MB, hit ratio %.2f)\n", window / 1e6,
                maxPersist / 1e6, v.accessPolicyWindow.hitRatio);
}

TraversalBuild buildTraversal(const dk_scene* sc, bool watertight) {
    // Traversal BVH: a binned-SAH tree over the triangles the caller's BVH
    // reaches, each carrying its reference DFS slot as the tie-break key.
    const double t0 = traceCreate() ? wallMs() : 0.0;
    struct Report {
        double t0;
        ~Report() {
            if (traceCreate()) fprintf(stderr, "[dk create] traversal build %.1f ms\n", wallMs() - t0);
        }
    } report{t0};
    TraversalBuild t;
    // The watertight mode's robust box test is the 4-wide tree's.
    t.width = watertight ? 4 : traversalWidth();
    std::vector<uint32_t> slotOf;
    std::string err;
    if (!referenceSlots(sc, slotOf, err)) {
        t.rc = DK_ERROR_INVALID_SCENE;
        t.err = "Invalid render scene: " + err + ".";
        return t;
    }
    if (traceCreate()) fprintf(stderr, "[dk create]   reference slots %.1f ms\n", wallMs() - t0);
    std::vector<uint8_t> opaque(sc->triangle_count);
    for (uint32_t i = 0; i < sc->triangle_count; ++i) {
        const dk_material& m = sc->materials[std::min(sc->triangles[i].material_id, sc->material_count - 1)];
        // shadowOccluded (PathTrace.metal:4230-4241): cut-outs pass, transmissive layers tint.
        opaque[i] = materialBlocksShadow(m) ? 1 : 0;
        if (!opaque[i] && slotOf[i] != kNoSlot) t.allOpaque = false;
    }
    t.rc = buildSahTraversal(sc, slotOf, opaque, t.width, t.nodes, t.isect, err);
    if (t.rc != DK_OK) {
        t.err = "Invalid render scene: " + err + ".";
        return t;
    }
    if (watertight) {
        // The watertight test reads the exact vertices: rows 1 and 2 of every
        // slot become v1 and v2 (the dummy slot stays degenerate).
        t.watertight = true;
        const size_t slots = t.isect.size() / 3;
        for (size_t k = 0; k < slots; ++k) {
            uint32_t slot, tri;
            std::memcpy(&slot, &t.isect[3 * k].w, 4);
            std::memcpy(&tri, &t.isect[3 * k + 1].w, 4);
            if (slot == 0xffffffffu || tri >= sc->triangle_count) continue;
            const dk_triangle& tr = sc->triangles[tri];
            t.isect[3 * k + 1] = make_float4(tr.v1.x, tr.v1.y, tr.v1.z, t.isect[3 * k + 1].w);
            t.isect[3 * k + 2] = make_float4(tr.v2.x, tr.v2.y, tr.v2.z, t.isect[3 * k + 2].w);
        }
    }
    return t;
}

int uploadScene(Arena& arena, const dk_scene* sc, DevScene& D, uint32_t materialCapacity,
                std::future<TraversalBuild>* pending) {
    // The traversal tree is built on another thread (`pending`, started by
    // the caller before its own allocations) or here; the other arrays are
    // uploaded meanwhile.
    std::future<TraversalBuild> local;
    if (!pending) {
        local = std::async(std::launch::async, [sc] { return buildTraversal(sc); });
        pending = &local;
    }
    struct Wait {  // the build reads `sc`: it must end before this returns
        std::future<TraversalBuild>* f;
        ~Wait() {
            if (f->valid()) f->wait();
        }
    } wait{pending};
    std::memset(&D, 0, sizeof(D));
#define TRY(x)                         \
    do {                               \
        int _rc = (x);                 \
        if (_rc != DK_OK) return _rc;  \
    } while (0)
    TRY(arena.upload(const_cast<dk_triangle**>(&D.tris), sc->triangles, sc->triangle_count, "triangles"));
    {
        dk_material* mats = nullptr;
        TRY(arena.alloc(&mats, std::max(materialCapacity, sc->material_count), "materials"));
        DK_CUDA(cudaMemcpy(mats, sc->materials, sc->material_count * sizeof(dk_material), cudaMemcpyHostToDevice),
                "materials");
        D.mats = mats;
    }
    TRY(arena.upload(const_cast<dk_texture_descriptor**>(&D.texdesc), sc->texture_descriptors,
                     sc->texture_descriptor_count, "texture descriptors"));
    TRY(arena.upload(const_cast<float4**>(&D.texpix), reinterpret_cast<const float4*>(sc->texture_pixels),
                     (size_t)sc->texture_pixel_count, "texture pixels"));
    TRY(arena.upload(const_cast<dk_light_record**>(&D.lights), sc->lights, sc->light_count, "lights"));
    TRY(arena.upload(const_cast<float2**>(&D.env), reinterpret_cast<const float2*>(sc->environment_samples),
                     sc->environment_sample_count, "environment samples"));
    // Guide table over the environment CDF (only when the CDF is monotone).
    if (sc->environment_sample_count > 1 && sc->environment_samples) {
        const uint32_t n = sc->environment_sample_count;
        bool monotone = true;
        for (uint32_t i = 1; i < n && monotone; ++i)
            monotone = sc->environment_samples[i].cdf >= sc->environment_samples[i - 1].cdf;
        if (monotone) {
            // One bucket per texel or finer (a power of two >= n, 2^13..2^22),
            // so the search after the guide lookup takes one or two steps.
            uint32_t G = 8192;
            while (G < n && G < (1u << 22)) G <<= 1;
            std::vector<uint32_t> guide(G + 1);
            uint32_t i = 0;
            for (uint32_t b = 0; b <= G; ++b) {
                float target = (float)b / (float)G;  // exact: b * 2^-log2(G)
                while (i < n && !(target <= sc->environment_samples[i].cdf)) ++i;
                guide[b] = i;  // first index with target <= cdf (n if none)
            }
            TRY(arena.upload(const_cast<uint32_t**>(&D.env_guide), guide.data(), guide.size(), "environment guide"));
            D.env_guide_size = G;
        }
    }
    // Sparse distance volumes: the reference arrays plus a distance-only copy
    // of the packed samples for the march.
    if (sc->volume_count) {
        TRY(arena.upload(const_cast<dk_volume_descriptor**>(&D.volumes), sc->volumes, sc->volume_count, "volumes"));
        TRY(arena.upload(const_cast<dk_volume_brick_descriptor**>(&D.bricks), sc->volume_bricks,
                         sc->volume_brick_count, "volume bricks"));
        TRY(arena.upload(const_cast<dk_volume_brick_sample**>(&D.brick_samples), sc->volume_brick_samples,
                         (size_t)sc->volume_brick_sample_count, "volume brick samples"));
        // FP16 (2 bytes a sample) when every stored distance is a half value
        // (a build with fp16_distances), else FP32: the same floats either way.
        const size_t ns = (size_t)sc->volume_brick_sample_count;
        std::vector<uint16_t> half(ns);
        bool halfExact = true;
        for (size_t i = 0; i < ns && halfExact; ++i) {
            const float d = sc->volume_brick_samples[i].distance;
            const __half h = __float2half_rn(d);
            halfExact = __half2float(h) == d && std::isfinite(d);
            half[i] = __half_as_ushort(h);
        }
        if (halfExact && ns > 0) {
            TRY(arena.upload(const_cast<uint16_t**>(&D.brick_dist16), half.data(), ns, "volume brick distances (FP16)"));
        } else {
            std::vector<float> dist(ns);
            for (size_t i = 0; i < ns; ++i) dist[i] = sc->volume_brick_samples[i].distance;
            TRY(arena.upload(const_cast<float**>(&D.brick_dist), dist.data(), dist.size(), "volume brick distances"));
        }
        TRY(arena.upload(const_cast<dk_volume_brick_grid**>(&D.brick_grids), sc->volume_brick_grids,
                         sc->volume_brick_grid_count, "volume brick grids"));
        TRY(arena.upload(const_cast<uint32_t**>(&D.brick_grid_indices), sc->volume_brick_grid_indices,
                         (size_t)sc->volume_brick_grid_index_count, "volume brick grid indices"));
        D.volume_count = sc->volume_count;
        D.brick_count = sc->volume_brick_count;
        D.brick_sample_count = sc->volume_brick_sample_count;
        D.brick_grid_count = sc->volume_brick_grid_count;
        D.brick_grid_index_count = sc->volume_brick_grid_index_count;
        bool volOpaque = true;
        for (uint32_t i = 0; i < sc->material_count; ++i)
            if (!materialBlocksShadow(sc->materials[i])) volOpaque = false;
        D.volume_all_opaque = volOpaque ? 1u : 0u;
    }
    {
        TraversalBuild t = pending->get();
        if (t.rc != DK_OK) return fail(t.rc, t.err);
        // Triangle slots and nodes in one block: the traversal working set is
        // one address range (an L2 access-policy window covers it).
        // Nodes start on a 128-byte line (a 4-wide node is one line).
        const size_t nodeOfs = (t.isect.size() + 7) / 8 * 8;
        float4* block = nullptr;
        TRY(arena.alloc(&block, nodeOfs + t.nodes.size(), "triangle slots + BVH nodes"));
        if (!t.isect.empty())
            DK_CUDA(cudaMemcpy(block, t.isect.data(), t.isect.size() * sizeof(float4), cudaMemcpyHostToDevice),
                    "triangle slots");
        if (!t.nodes.empty())
            DK_CUDA(cudaMemcpy(block + nodeOfs, t.nodes.data(), t.nodes.size() * sizeof(float4),
                               cudaMemcpyHostToDevice),
                    "BVH nodes");
        D.isect = block;
        D.nodes = block + nodeOfs;
        D.traversal_bytes = (nodeOfs + t.nodes.size()) * sizeof(float4);
        D.node_count = (uint32_t)(t.nodes.size() / (t.width == 8 ? 5 : 8));
        D.wide8 = t.width == 8 ? 1u : 0u;
        D.watertight = t.watertight ? 1u : 0u;
        D.all_shadow_opaque = t.allOpaque ? 1u : 0u;
    }
#undef TRY
    D.tri_count = sc->triangle_count;
    D.mat_count = sc->material_count;
    D.texdesc_count = sc->texture_descriptor_count;
    D.light_count = sc->lights ? sc->light_count : 0;
    D.env_count = sc->environment_samples ? sc->environment_sample_count : 0;
    D.env_tex_plus1 = sc->environment_texture_index_plus_one;
    D.env_intensity = sc->environment_intensity;
    D.env_rot_y = sc->environment_rotation_y;
    {
        float* dsc = nullptr;
        int rc = arena.alloc(&dsc, 2, "environment rotation");
        if (rc != DK_OK) return rc;
        DK_CUDA(envRotation(D.env_rot_y, dsc, 0), "environment rotation");
        float hsc[2];
        DK_CUDA(cudaMemcpy(hsc, dsc, sizeof(hsc), cudaMemcpyDeviceToHost), "environment rotation");
        D.env_rot_sin = hsc[0];
        D.env_rot_cos = hsc[1];
    }
    D.env_max_radiance = sc->environment_max_radiance;
    return DK_OK;
}

int allocWave(Arena& arena, Wave& W, uint64_t capPaths, uint32_t pixelCap, uint32_t jobCap) {
    std::memset(&W, 0, sizeof(W));
    W.cap = (uint32_t)capPaths;
    W.aov_stride = pixelCap;
    const size_t cap = W.cap;
#define TRY(x)                         \
    do {                               \
        int _rc = (x);                 \
        if (_rc != DK_OK) return _rc;  \
    } while (0)
    TRY(arena.alloc(&W.ray_o, cap, "ray origins"));
    TRY(arena.alloc(&W.ray_d, cap, "ray directions"));
    TRY(arena.alloc(&W.tp, cap, "throughput"));
    TRY(arena.alloc(&W.rad, cap, "radiance"));
    TRY(arena.alloc(&W.rng, cap, "rng"));
    TRY(arena.alloc(&W.hit, cap, "hits"));
    TRY(arena.alloc(&W.nee_o, 3 * cap, "shadow origins"));
    TRY(arena.alloc(&W.nee_d, 3 * cap, "shadow directions"));
    TRY(arena.alloc(&W.nee_c, 3 * cap, "shadow contributions"));
    TRY(arena.alloc(&W.nee_tp, cap, "shadow throughput"));
    TRY(arena.alloc(&W.q[0], cap, "queue 0"));
    TRY(arena.alloc(&W.q[1], cap, "queue 1"));
    TRY(arena.alloc(&W.qs, cap, "shadow queue"));
    TRY(arena.alloc(&W.qr, 3 * cap, "shadow ray queue"));
    TRY(arena.alloc(&W.qr2, 3 * cap, "layer-walk queue"));
    TRY(arena.alloc(&W.counts, 16, "queue counters"));
    TRY(arena.alloc(&W.aov, 4 * (size_t)pixelCap, "AOV records"));
    TRY(arena.alloc(&W.layer_hits, 3 * cap * kRecLayers, "recorded shadow layers"));
    TRY(arena.alloc(&W.layer_count, 3 * cap, "recorded shadow layer counts"));
    TRY(arena.alloc(&W.live, cap, "survivor flags"));
    TRY(arena.alloc(&W.scan, (cap + kLiveBlock - 1) / kLiveBlock + 1, "survivor block offsets"));
    TRY(arena.alloc(&W.qsorted, cap, "material-ordered queue"));
    TRY(arena.alloc(&W.keys, cap, "material keys"));
    TRY(arena.alloc(&W.bins, kSortBins + 1, "material bins"));
    DevJob* jobs = nullptr;
    TRY(arena.alloc(&jobs, std::max(jobCap, 1u), "job table"));
    W.jobs = jobs;
#undef TRY
    return DK_OK;
}

int allocAccum(Arena& arena, Accum& A, size_t pixels) {
    std::memset(&A, 0, sizeof(A));
    int rc;
    if ((rc = arena.alloc(&A.sum, pixels, "accumulation sum")) != DK_OK) return rc;
    if ((rc = arena.alloc(&A.comp, pixels, "accumulation compensation")) != DK_OK) return rc;
    if ((rc = arena.alloc(&A.resolved, pixels, "accumulation resolve")) != DK_OK) return rc;
    if ((rc = arena.alloc(&A.count, pixels, "sample counts")) != DK_OK) return rc;
    return arena.alloc(&A.aov, 6 * pixels, "AOV planes");
}

int clearAccum(const Accum& A, size_t pixels, cudaStream_t st) {
    DK_CUDA(cudaMemsetAsync(A.sum, 0, pixels * sizeof(float4), st), "clear accumulation");
    DK_CUDA(cudaMemsetAsync(A.comp, 0, pixels * sizeof(float4), st), "clear accumulation");
    DK_CUDA(cudaMemsetAsync(A.resolved, 0, pixels * sizeof(D4), st), "clear accumulation");
    DK_CUDA(cudaMemsetAsync(A.count, 0, pixels * sizeof(uint32_t), st), "clear accumulation");
    return DK_OK;
}

void fillParams(DevParams& P, const dk_settings& st) {
    std::memset(&P, 0, sizeof(P));
    P.width = st.width;
    P.height = st.height;
    P.max_bounces = std::max(1u, st.max_bounces);
    P.transparent_background = st.transparent_background;
    P.shows_env_bg = st.shows_environment_background;
    P.frame_seed = st.frame_seed;
    P.denoiser = st.denoiser_enabled;
    P.bg[0] = st.background_color[0];
    P.bg[1] = st.background_color[1];
    P.bg[2] = st.background_color[2];
    P.clamp = st.sample_radiance_clamp_set ? st.sample_radiance_clamp : 64.0f;  // RenderQuality.final default
    P.tile_x = 0;
    P.tile_y = 0;
    P.tile_w = st.width;
    P.tile_h = st.height;
    P.cam = st.camera;
    P.prev_cam = st.previous_camera;
}

int launchWave(const DevScene& S, const Wave& W, uint32_t maxBounces, bool anyDenoiser, const Grids& g,
               cudaStream_t q, const std::function<int(int)>& mark, uint64_t& launches) {
#define MARK(k)                       \
    do {                              \
        int _rc = mark(k);            \
        if (_rc != DK_OK) return _rc; \
    } while (0)
    MARK(0);
    DK_CUDA(launchGenerate(S, W, g.gen, q), "generate launch");
    ++launches;
    for (uint32_t b = 0; b < maxBounces; ++b) {
        uint32_t sel = b & 1u;
        MARK(1);
        DK_CUDA(launchExtend(S, W, sel, b, S.wide8 ? g.extend8 : g.extend, g.volume, q), "extend launch");
        MARK(2);
        DK_CUDA(launchShade(S, W, b, sel, g.shade, q), "shade launch");
        MARK(3);
        DK_CUDA(launchShadow(S, W, S.wide8 ? g.shadow8 : g.shadow, q), "shadow launch");
        DK_CUDA(launchResolve(W, g.final, q), "resolve launch");
        launches += bounceLaunches(S);
    }
    MARK(0);
    if (anyDenoiser) {
        DK_CUDA(launchAovPrimary(S, W, g.extend, q), "AOV launch");
        ++launches;
    }
    DK_CUDA(launchFinalize(W, g.final, q), "finalize launch");
    ++launches;
    MARK(0);
#undef MARK
    return DK_OK;
}

}  // namespace dk

extern "C" {

const char* dk_last_error_message(void) { return dk::lastError(); }

const char* dk_version(void) { return "denrim-gb300 0.1 (sm_103a wavefront path tracer)"; }

int dk_device_count(int* out) {
    if (!out) return fail(DK_ERROR_INVALID_ARGUMENT, "out_count is null");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *out = n;
    return DK_OK;
}

int dk_device_open(int ordinal) { return dk::openDevice(ordinal); }

int dk_build_bvh(const dk_triangle* tris, uint32_t n, uint32_t maxLeaf, dk_bvh_node* nodes, uint32_t* nodeCount,
                 uint32_t* primIdx) {
    if (!nodeCount || (n > 0 && (!tris || !nodes || !primIdx)))
        return fail(DK_ERROR_INVALID_ARGUMENT, "dk_build_bvh: null argument");
    *nodeCount = buildReferenceBvh(tris, n, maxLeaf, nodes, primIdx);
    return DK_OK;
}

int dk_build_lights(dk_triangle* tris, uint32_t n, const dk_material* mats, uint32_t matCount,
                    dk_light_record* lights, uint32_t* lightCount) {
    if (!lightCount || (n > 0 && (!tris || !lights)) || (matCount > 0 && !mats))
        return fail(DK_ERROR_INVALID_ARGUMENT, "dk_build_lights: null argument");
    *lightCount = 0;
    if (matCount == 0) return DK_OK;
    // lightRecordsAndTaggedTriangles (LightingGPUEncoding.swift:5-64).
    struct C { uint32_t tri, mat; float area, weight, nx, ny, nz; };
    std::vector<C> cands;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t mi = std::min(tris[i].material_id, matCount - 1);
        const dk_float4& e = mats[mi].emission;
        if (!(std::fmax(std::fmax(e.x, e.y), e.z) > 0.0f)) continue;
        float ax = tris[i].v1.x - tris[i].v0.x, ay = tris[i].v1.y - tris[i].v0.y, az = tris[i].v1.z - tris[i].v0.z;
        float bx = tris[i].v2.x - tris[i].v0.x, by = tris[i].v2.y - tris[i].v0.y, bz = tris[i].v2.z - tris[i].v0.z;
        float cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
        float len = std::sqrt(cx * cx + cy * cy + cz * cz);
        float area = len * 0.5f;
        if (!(area > 0.0f)) continue;
        float power = (e.x * 0.2126f + e.y * 0.7152f + e.z * 0.0722f) * area;
        if (!(power > 0.0f)) continue;
        float s = 1.0f / len;
        cands.push_back({i, mi, area, power, cx * s, cy * s, cz * s});
    }
    float total = 0.0f;
    for (auto& c : cands) total += c.weight;
    if (!(total > 0.0f)) return DK_OK;
    float cum = 0.0f;
    for (size_t k = 0; k < cands.size(); ++k) {
        cum += cands[k].weight;
        tris[cands[k].tri].padding2 = (uint32_t)(k + 1);
        lights[k].triangle_index = cands[k].tri;
        lights[k].material_index = cands[k].mat;
        lights[k].area = cands[k].area;
        lights[k].selection_cdf = (k == cands.size() - 1) ? 1.0f : std::fmin(cum / total, 1.0f);
        lights[k].normal = {cands[k].nx, cands[k].ny, cands[k].nz, 0.0f};
    }
    *lightCount = (uint32_t)cands.size();
    return DK_OK;
}

int dk_build_environment_samples(const dk_float4* pixels, uint32_t w, uint32_t h, float intensity, float maxRadiance,
                                 dk_environment_sample* out, uint32_t* outCount) {
    if (!outCount || (w > 0 && h > 0 && (!pixels || !out)))
        return fail(DK_ERROR_INVALID_ARGUMENT, "dk_build_environment_samples: null argument");
    *outCount = 0;
    if (w == 0 || h == 0) return DK_OK;
    int rc = dk::ensureDevice();
    if (rc != DK_OK) return rc;
    size_t n = (size_t)w * h;
    if (n > 0xffffffffull / 2) return fail(DK_ERROR_INVALID_ARGUMENT, "environment map too large");
    uint32_t nb = (uint32_t)((n + 1023) / 1024);
    float4* dPix = nullptr;
    double *dW = nullptr, *dP = nullptr, *dB = nullptr;
    float2* dOut = nullptr;
    cudaError_t e = cudaMalloc(&dPix, n * sizeof(float4));
    if (e == cudaSuccess) e = cudaMalloc(&dW, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dP, n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dB, (nb + 1) * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dOut, n * sizeof(float2));
    double total = 0.0;
    if (e == cudaSuccess) e = cudaMemcpy(dPix, pixels, n * sizeof(float4), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = dk::buildEnvironmentTable(dPix, w, h, std::fmax(intensity, 0.0f), std::fmax(maxRadiance, 0.0f), dW, dP, dB,
                                      dOut, 4 * dk::deviceProp().multiProcessorCount, 0, &total);
    if (e == cudaSuccess && total > 0.0) e = cudaMemcpy(out, dOut, n * sizeof(float2), cudaMemcpyDeviceToHost);
    cudaFree(dPix);
    cudaFree(dW);
    cudaFree(dP);
    cudaFree(dB);
    cudaFree(dOut);
    if (e != cudaSuccess) return fail(DK_ERROR_COMMAND_FAILED, std::string("environment table: ") + cudaGetErrorString(e));
    *outCount = total > 0.0 ? (uint32_t)n : 0u;
    return DK_OK;
}

int dk_session_create(const dk_scene* sc, const dk_settings* st, dk_session** outSession) {
    if (!sc || !st || !outSession) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_session_create: null argument");
    *outSession = nullptr;
    // RenderSession.init validation (RenderSession.swift:304-327).
    if (st->width == 0 || st->height == 0)
        return fail(DK_ERROR_INVALID_SCENE, "Invalid render scene: Render dimensions must be positive.");
    if (st->quality > DK_QUALITY_FINAL) return fail(DK_ERROR_INVALID_ARGUMENT, "unknown render quality");
    if (st->triangle_test > DK_TRIANGLE_TEST_WATERTIGHT)
        return fail(DK_ERROR_INVALID_ARGUMENT, "unknown triangle test");
    int rc = dk::validateScene(sc);
    if (rc != DK_OK) return rc;
    rc = dk::ensureDevice();
    if (rc != DK_OK) return rc;
    const bool trace = dk::traceCreate();
    double tPrev = trace ? dk::wallMs() : 0.0;
    auto phase = [&](const char* what) {
        if (!trace) return;
        double now = dk::wallMs();
        fprintf(stderr, "[dk create] %s %.1f ms\n", what, now - tPrev);
        tPrev = now;
    };
    // The host traversal build runs while this thread allocates the wave.
    const bool watertight = st->triangle_test == DK_TRIANGLE_TEST_WATERTIGHT;
    std::future<dk::TraversalBuild> traversal =
        std::async(std::launch::async, [sc, watertight] { return dk::buildTraversal(sc, watertight); });
    struct WaitBuild {  // the build reads `sc`: it must end before this returns
        std::future<dk::TraversalBuild>& f;
        ~WaitBuild() {
            if (f.valid()) f.wait();
        }
    } waitBuild{traversal};

    Session* s = new Session();
    std::memset(&s->stats, 0, sizeof(s->stats));
    s->settings = *st;
    if (s->settings.max_bounces < 1) s->settings.max_bounces = 1;
#define TRY(x)                 \
    do {                       \
        int _rc = (x);         \
        if (_rc != DK_OK) {    \
            freeSession(s);    \
            return _rc;        \
        }                      \
    } while (0)
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess) {
        freeSession(s);
        return fail(DK_ERROR_COMMAND_FAILED, "cudaStreamCreate failed");
    }
    // Wave capacity: whole frames of the tile, up to a fixed path budget.
    const uint32_t pixels = st->width * st->height;
    uint64_t capPaths = 1ull << 24;  // 16.8 M paths (~3.5 GB of path state)
    if (st->max_samples_per_launch > 0) capPaths = std::min<uint64_t>(capPaths, (uint64_t)st->max_samples_per_launch * pixels);
    capPaths = std::max<uint64_t>(capPaths, pixels);
    capPaths = std::min<uint64_t>(capPaths, 1ull << 29);  // path indices fit 29 bits of the NEE record
    phase("stream");
    if (st->quality == DK_QUALITY_FINAL) {  // preview / interactive keep no path state
        TRY(dk::allocWave(s->arena, s->wave, capPaths, pixels, 1));
        s->jobs = const_cast<dk::DevJob*>(s->wave.jobs);
    }
    phase("wave allocation");
    TRY(dk::allocAccum(s->arena, s->accum, pixels));
    TRY(s->arena.alloc(&s->staging, pixels, "readback staging"));
    phase("accumulation allocation");
    TRY(dk::uploadScene(s->arena, sc, s->scene, sc->material_count, &traversal));
    phase("scene upload (with the traversal build's tail)");
    if (st->collects_traversal_stats) {  // RenderSettings.collectsSDFTraversalStats (RenderSettings.swift:73)
        TRY(s->arena.alloc(&s->sdfCounters, dk::kSdfCounterSlots, "SDF traversal counters"));
        s->scene.sdf_counters = s->sdfCounters;
        if (cudaMemsetAsync(s->sdfCounters, 0, dk::kSdfCounterSlots * sizeof(unsigned long long), s->stream) !=
            cudaSuccess) {
            freeSession(s);
            return fail(DK_ERROR_COMMAND_FAILED, "clearing the SDF traversal counters failed");
        }
    }
    dk::persistTraversal(s->scene, s->stream);
    s->opaqueMask = dk::opaqueMask(sc->materials, sc->material_count);
    TRY(dk::clearAccum(s->accum, pixels, s->stream));
    if (cudaMemsetAsync(s->accum.aov, 0, 6 * (size_t)pixels * sizeof(float4), s->stream) != cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess) {
        freeSession(s);
        return fail(DK_ERROR_COMMAND_FAILED, "clearing accumulation buffers failed");
    }
    s->grids = dk::kernelGrids();
    s->stats.device_bytes = s->arena.bytes;
    phase("clears");
    *outSession = reinterpret_cast<dk_session*>(s);
    return DK_OK;
#undef TRY
}

static int eventAt(Session* s, size_t i, cudaEvent_t* out) {
    while (s->evPool.size() <= i) {
        cudaEvent_t e;
        DK_CUDA(cudaEventCreate(&e), "cudaEventCreate");
        s->evPool.push_back(e);
    }
    *out = s->evPool[i];
    return DK_OK;
}

// Renders `samples` sample indices starting at `sampleBegin` over a tile, in
// batches of whole tile-frames that fit the wave (a one-job wave each).  Every
// stage is bracketed by events on the session stream; they are read once,
// after the last batch.
// RenderQuality.preview / .interactive: the kernel overwrites the tile's
// beauty and AOVs on every sample and ignores the sample index, so one pass
// stands for any number of samples.
static int renderPreview(Session* s, uint32_t tx, uint32_t ty, uint32_t tw, uint32_t th, uint32_t samples) {
    const dk_settings& st = s->settings;
    dk::DevParams P;
    dk::fillParams(P, st);
    P.tile_x = tx;
    P.tile_y = ty;
    P.tile_w = tw;
    P.tile_h = th;
    P.samples_in_batch = 1;
    cudaEvent_t e0, e1;
    int rc = eventAt(s, 0, &e0);
    if (rc == DK_OK) rc = eventAt(s, 1, &e1);
    if (rc != DK_OK) return rc;
    DK_CUDA(cudaEventRecord(e0, s->stream), "cudaEventRecord");
    DK_CUDA(dk::launchPreview(s->scene, P, s->accum, s->scene.mat_count, s->opaqueMask,
                              st.quality == DK_QUALITY_INTERACTIVE, s->grids.extend, s->stream),
            "preview launch");
    DK_CUDA(cudaEventRecord(e1, s->stream), "cudaEventRecord");
    DK_CUDA(cudaEventSynchronize(e1), "render");
    float ms = 0;
    DK_CUDA(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
    s->stats.last_render_ms = ms;
    s->stats.last_extend_ms = s->stats.last_shade_ms = s->stats.last_shadow_ms = 0;
    s->stats.last_other_ms = ms;
    s->stats.last_launches = 1;
    s->stats.kernel_launches += 1;
    s->stats.paths_traced += (uint64_t)tw * th * samples;
    return DK_OK;
}

static int renderSamples(Session* s, uint32_t tx, uint32_t ty, uint32_t tw, uint32_t th, uint32_t samples,
                         uint32_t sampleBegin) {
    const dk_settings& st = s->settings;
    if (st.quality != DK_QUALITY_FINAL) return renderPreview(s, tx, ty, tw, th, samples);
    dk::DevJob job;
    std::memset(&job, 0, sizeof(job));
    dk::fillParams(job.P, st);
    job.P.tile_x = tx;
    job.P.tile_y = ty;
    job.P.tile_w = tw;
    job.P.tile_h = th;
    job.A = s->accum;
    job.mat_base = 0;
    job.mat_count = s->scene.mat_count;
    job.opaque_mask = s->opaqueMask;
    const uint32_t tileN = tw * th;
    const uint32_t perBatch = std::max(1u, s->wave.cap / tileN);
    cudaStream_t q = s->stream;
    // Event marks: kind 0 = other, 1 = extend, 2 = shade, 3 = shadow; the
    // interval between mark i and mark i+1 belongs to kind[i].
    std::vector<int> kinds;
    size_t ev = 0;
    bool capturing = false;
    auto mark = [&](int kind) -> int {
        cudaEvent_t e;
        int rc = eventAt(s, ev++, &e);
        if (rc != DK_OK) return rc;
        // Under stream capture the record must be external to become a node
        // of the graph (recorded on every replay); the flag is refused on an
        // ordinary record.
        DK_CUDA(capturing ? cudaEventRecordWithFlags(e, q, cudaEventRecordExternal) : cudaEventRecord(e, q),
                "cudaEventRecord");
        kinds.push_back(kind);
        return DK_OK;
    };
    uint64_t launches = 0;
    uint32_t done = 0;
    // A render of one wave runs as a CUDA graph (DK_RENDER_GRAPHS=0: plain
    // launches): the job table is uploaded on the stream as usual, then the
    // captured kernel sequence of the wave is replayed.
    static const bool useGraphs = [] {
        const char* e = getenv("DK_RENDER_GRAPHS");
        return !(e && e[0] == '0');
    }();
    if (useGraphs && samples <= perBatch) {
        const uint32_t nb = samples;
        job.P.sample_begin = sampleBegin;
        job.P.samples_in_batch = nb;
        job.P.path_count = nb * tileN;
        DK_CUDA(cudaMemcpyAsync(s->jobs, &job, sizeof(job), cudaMemcpyHostToDevice, q), "job table upload");
        Session::WaveGraph* g = nullptr;
        for (auto& c : s->graphs)
            if (c.tx == tx && c.ty == ty && c.tw == tw && c.th == th && c.nb == nb &&
                c.bounces == job.P.max_bounces && c.aovs == (st.denoiser_enabled != 0))
                g = &c;
        if (!g && !s->graphsFailed) {
            // Events the capture records into (created beforehand: no
            // allocation while capturing).
            cudaEvent_t e;
            int rc = eventAt(s, 4 * (size_t)job.P.max_bounces + 8, &e);
            if (rc != DK_OK) return rc;
            dk::Wave W = s->wave;
            W.job_count = 1;
            W.path_count = job.P.path_count;
            W.pixel_count = tileN;
            uint64_t n = 0;
            cudaGraph_t graph = nullptr;
            cudaGraphExec_t exec = nullptr;
            bool ok = cudaStreamBeginCapture(q, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
            if (ok) {
                capturing = true;
                rc = dk::launchWave(s->scene, W, job.P.max_bounces, st.denoiser_enabled != 0, s->grids, q, mark, n);
                capturing = false;
                ok = cudaStreamEndCapture(q, &graph) == cudaSuccess && rc == DK_OK && graph &&
                     cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
            }
            if (graph) cudaGraphDestroy(graph);
            if (ok) {
                s->graphs.push_back({tx, ty, tw, th, nb, job.P.max_bounces, st.denoiser_enabled != 0, exec, ev,
                                     kinds, n});
                g = &s->graphs.back();
            } else {  // capture refused: plain launches for this session
                cudaGetLastError();
                s->graphsFailed = true;
                ev = 0;
                kinds.clear();
            }
        }
        if (g) {
            DK_CUDA(cudaGraphLaunch(g->exec, q), "graph launch");
            ev = g->events;
            kinds = g->kinds;
            launches = g->launches;
            done = samples;
        }
    }
    while (done < samples) {
        uint32_t nb = std::min(perBatch, samples - done);
        job.P.sample_begin = sampleBegin + done;
        job.P.samples_in_batch = nb;
        job.P.path_count = nb * tileN;
        // Pageable source: the copy is staged before the call returns, so
        // `job` may change for the next batch at once.
        DK_CUDA(cudaMemcpyAsync(s->jobs, &job, sizeof(job), cudaMemcpyHostToDevice, q), "job table upload");
        dk::Wave W = s->wave;
        W.job_count = 1;
        W.path_count = job.P.path_count;
        W.pixel_count = tileN;
        int rc = dk::launchWave(s->scene, W, job.P.max_bounces, st.denoiser_enabled != 0, s->grids, q, mark, launches);
        if (rc != DK_OK) return rc;
        done += nb;
    }
    DK_CUDA(cudaEventSynchronize(s->evPool[ev - 1]), "render");
    float t[4] = {0, 0, 0, 0};
    for (size_t i = 0; i + 1 < ev; ++i) {
        float ms = 0;
        DK_CUDA(cudaEventElapsedTime(&ms, s->evPool[i], s->evPool[i + 1]), "cudaEventElapsedTime");
        t[kinds[i]] += ms;
    }
    float total = 0;
    DK_CUDA(cudaEventElapsedTime(&total, s->evPool[0], s->evPool[ev - 1]), "cudaEventElapsedTime");
    s->stats.last_render_ms = total;
    s->stats.last_extend_ms = t[1];
    s->stats.last_shade_ms = t[2];
    s->stats.last_shadow_ms = t[3];
    s->stats.last_other_ms = t[0];
    s->stats.last_launches = launches;
    s->stats.kernel_launches += launches;
    s->stats.paths_traced += (uint64_t)tileN * samples;
    return DK_OK;
}

int dk_session_render(dk_session* session, uint32_t samples) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "session is null");
    if (samples == 0) return DK_OK;
    int rc = renderSamples(s, 0, 0, s->settings.width, s->settings.height, samples, s->sampleCount);
    if (rc != DK_OK) {
        cudaGetLastError();
        return rc;  // sampleCount unchanged (RenderSession.swift:844-847)
    }
    s->sampleCount += samples;
    return DK_OK;
}

int dk_session_render_tile(dk_session* session, uint32_t x, uint32_t y, uint32_t w, uint32_t h, int completes) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "session is null");
    // encodeNextSample tile clamping (RenderSession.swift:898-907).
    uint32_t W = s->settings.width, H = s->settings.height;
    uint32_t tx = std::min(x, W), ty = std::min(y, H);
    uint32_t tw = std::min(w, W - tx), th = std::min(h, H - ty);
    if (tw == 0 || th == 0) return DK_OK;
    int rc = renderSamples(s, tx, ty, tw, th, 1, s->sampleCount);
    if (rc != DK_OK) {
        cudaGetLastError();
        return rc;
    }
    if (completes) s->sampleCount += 1;
    return DK_OK;
}

int dk_session_update_camera(dk_session* session, const dk_camera* camera, const dk_camera* previous) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s || !camera) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    dk_camera old = s->settings.camera;
    s->settings.camera = *camera;
    s->settings.previous_camera = previous ? *previous : old;
    return dk_session_reset(session);
}

int dk_session_reset(dk_session* session) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "session is null");
    size_t pixels = (size_t)s->settings.width * s->settings.height;
    int rc = dk::clearAccum(s->accum, pixels, s->stream);
    if (rc != DK_OK) return rc;
    DK_CUDA(cudaStreamSynchronize(s->stream), "reset");
    s->sampleCount = 0;
    return DK_OK;
}

// The output plane `output` of the session on the device (the resolved
// beauty in the staging buffer, or an AOV plane).
static int outputPlane(Session* s, int output, const float4** src) {
    const size_t pixels = (size_t)s->settings.width * s->settings.height;
    if (output < DK_OUTPUT_BEAUTY || output > DK_OUTPUT_MOTION_VECTOR)
        return fail(DK_ERROR_INVALID_ARGUMENT, "unknown output kind");
    if (output == DK_OUTPUT_BEAUTY) {
        DK_CUDA(dk::launchResolveBeauty(s->accum, (uint32_t)pixels, s->staging, s->grids.final, s->stream), "resolve launch");
        *src = s->staging;
    } else {
        *src = s->accum.aov + (size_t)(output - 1) * pixels;
    }
    return DK_OK;
}

int dk_session_read_output(dk_session* session, int output, float* rgba, size_t pixelCount) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s || !rgba) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    size_t pixels = (size_t)s->settings.width * s->settings.height;
    if (pixelCount != pixels) return fail(DK_ERROR_INVALID_ARGUMENT, "pixel_count must equal width*height");
    if (output < DK_OUTPUT_BEAUTY || output > DK_OUTPUT_MOTION_VECTOR)
        return fail(DK_ERROR_INVALID_ARGUMENT, "unknown output kind");
    const float4* src = nullptr;
    int rc = outputPlane(s, output, &src);
    if (rc != DK_OK) return rc;
    DK_CUDA(cudaMemcpyAsync(rgba, src, pixels * sizeof(float4), cudaMemcpyDeviceToHost, s->stream), "readback");
    DK_CUDA(cudaStreamSynchronize(s->stream), "readback");
    return DK_OK;
}

int dk_session_copy_output(dk_session* session, int output, void* deviceRgba, size_t pixelCount, void* stream) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s || !deviceRgba) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    const size_t pixels = (size_t)s->settings.width * s->settings.height;
    if (pixelCount != pixels) return fail(DK_ERROR_INVALID_ARGUMENT, "pixel_count must equal width*height");
    if (reinterpret_cast<uintptr_t>(deviceRgba) % 16u)
        return fail(DK_ERROR_INVALID_ARGUMENT, "device_rgba must be 16-byte aligned");
    const float4* src = nullptr;
    int rc = outputPlane(s, output, &src);
    if (rc != DK_OK) return rc;
    DK_CUDA(cudaMemcpyAsync(deviceRgba, src, pixels * sizeof(float4), cudaMemcpyDeviceToDevice, s->stream),
            "output copy");
    if (!stream) {
        DK_CUDA(cudaStreamSynchronize(s->stream), "output copy");
        return DK_OK;
    }
    if (!s->copyDone) DK_CUDA(cudaEventCreateWithFlags(&s->copyDone, cudaEventDisableTiming), "cudaEventCreate");
    DK_CUDA(cudaEventRecord(s->copyDone, s->stream), "cudaEventRecord");
    DK_CUDA(cudaStreamWaitEvent(static_cast<cudaStream_t>(stream), s->copyDone, 0), "cudaStreamWaitEvent");
    return DK_OK;
}

int dk_session_read_rgba8(dk_session* session, int output, uint8_t* rgba, size_t bytes) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s || !rgba) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    const size_t pixels = (size_t)s->settings.width * s->settings.height;
    if (bytes != pixels * 4) return fail(DK_ERROR_INVALID_ARGUMENT, "bytes must equal width*height*4");
    const float4* src = nullptr;
    int rc = outputPlane(s, output, &src);
    if (rc != DK_OK) return rc;
    if (!s->rgba8) {
        int arc = s->arena.alloc(&s->rgba8, pixels, "display bytes");
        if (arc != DK_OK) return arc;
        arc = s->arena.alloc(&s->encodeWs, DK_ENCODE_WORKSPACE_BYTES / sizeof(uint32_t), "display workspace");
        if (arc != DK_OK) return arc;
    }
    DK_CUDA(dk::encodeRgba8(src, (uint32_t)pixels, output, s->encodeWs, s->rgba8, s->stream), "encode launch");
    DK_CUDA(cudaMemcpyAsync(rgba, s->rgba8, bytes, cudaMemcpyDeviceToHost, s->stream), "readback");
    DK_CUDA(cudaStreamSynchronize(s->stream), "readback");
    return DK_OK;
}

int dk_session_write_png(dk_session* session, int output, const char* path) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s || !path) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    std::vector<uint8_t> bytes((size_t)s->settings.width * s->settings.height * 4);
    int rc = dk_session_read_rgba8(session, output, bytes.data(), bytes.size());
    if (rc != DK_OK) return rc;
    return dk::writePng(path, bytes.data(), s->settings.width, s->settings.height);
}

int dk_session_sample_count(const dk_session* session, uint32_t* out) {
    const Session* s = reinterpret_cast<const Session*>(session);
    if (!s || !out) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    *out = s->sampleCount;
    return DK_OK;
}

int dk_session_stats(const dk_session* session, dk_stats* out) {
    const Session* s = reinterpret_cast<const Session*>(session);
    if (!s || !out) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    *out = s->stats;
    if (s->sdfCounters) {  // sdfTraversalStats (RenderSession.swift:808-831)
        unsigned long long c[dk::kSdfCounterSlots];
        if (cudaStreamSynchronize(s->stream) != cudaSuccess ||
            cudaMemcpy(c, s->sdfCounters, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess)
            return fail(DK_ERROR_COMMAND_FAILED, "reading the SDF traversal counters failed");
        for (uint32_t k = 0; k < dk::kSdfCounterSlots; ++k) out->sdf_counters[k] = c[k];
    }
    return DK_OK;
}

int dk_session_reset_sdf_stats(dk_session* session) {
    Session* s = reinterpret_cast<Session*>(session);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    if (!s->sdfCounters) return DK_OK;
    if (cudaMemsetAsync(s->sdfCounters, 0, dk::kSdfCounterSlots * sizeof(unsigned long long), s->stream) != cudaSuccess ||
        cudaStreamSynchronize(s->stream) != cudaSuccess)
        return fail(DK_ERROR_COMMAND_FAILED, "clearing the SDF traversal counters failed");
    return DK_OK;
}

int dk_session_destroy(dk_session* session) {
    freeSession(reinterpret_cast<Session*>(session));
    return DK_OK;
}

}  // extern "C"
