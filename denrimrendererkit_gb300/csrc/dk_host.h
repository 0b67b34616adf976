// Host-side pieces shared by the session (dk_host.cu) and the serving loop
// (dk_server.cu): error reporting, device selection, device-memory arenas, the
// scene upload with the traversal-BVH conversion, wave and accumulation
// buffers, and the launch sequence of one wave.
#pragma once
#include <cstdint>
#include <functional>
#include <future>
#include <string>
#include <vector>

#include "dk_kernels.h"

namespace dk {

int fail(int code, const std::string& msg);  // records the message for dk_last_error_message
int ensureDevice();
const cudaDeviceProp& deviceProp();

#define DK_CUDA(call, what)                                                                                  \
    do {                                                                                                     \
        cudaError_t _e = (call);                                                                             \
        if (_e != cudaSuccess) {                                                                             \
            int _code = (_e == cudaErrorMemoryAllocation) ? DK_ERROR_OUT_OF_MEMORY : DK_ERROR_COMMAND_FAILED; \
            return ::dk::fail(_code, std::string(what) + ": " + cudaGetErrorString(_e));                      \
        }                                                                                                    \
    } while (0)

// Device allocations owned together and released together.
struct Arena {
    struct Buffer {
        void* ptr;
        size_t bytes;
    };
    std::vector<Buffer> buffers;
    size_t bytes = 0;

    int allocBytes(void** out, size_t bytes, const char* what);
    template <typename T>
    int alloc(T** out, size_t count, const char* what) {
        void* p = nullptr;
        int rc = allocBytes(&p, count * sizeof(T), what);
        *out = static_cast<T*>(p);
        return rc;
    }
    template <typename T>
    int upload(T** out, const T* host, size_t count, const char* what) {
        int rc = alloc(out, count, what);
        if (rc != DK_OK || count == 0) return rc;
        DK_CUDA(cudaMemcpy(*out, host, count * sizeof(T), cudaMemcpyHostToDevice), what);
        return DK_OK;
    }
    void release();
};

// RenderSession.init scene validation (RenderSession.swift:304-327) plus the
// ABI's pointer/count consistency checks.
int validateScene(const dk_scene* sc);

// Uploads `sc` into `D` (traversal BVH, environment guide table, sparse-volume
// arrays).  `materialCapacity` >= sc->material_count reserves room in D.mats
// for per-render material tables appended later.
// The traversal tree of a scene (host work, see dk_bvh.cu), built apart from
// the upload so that it can run while the caller allocates device memory.
struct TraversalBuild {
    int rc = DK_OK;
    std::string err;
    int width = 4;
    bool allOpaque = true;
    bool watertight = false;  // slot rows hold v1, v2 (watertight test) instead of the edges
    std::vector<float4> nodes, isect;
};
// `watertight`: the slots carry absolute vertices for the watertight test
// (dk_settings.triangle_test = DK_TRIANGLE_TEST_WATERTIGHT).
TraversalBuild buildTraversal(const dk_scene* sc, bool watertight = false);
// Uploads the scene; `pending` (may be null) is a traversal build already
// started with std::async(buildTraversal).
int uploadScene(Arena& arena, const dk_scene* sc, DevScene& D, uint32_t materialCapacity,
                std::future<TraversalBuild>* pending = nullptr);
// The traversal arrays as a persisting L2 window of `stream` (best effort).
void persistTraversal(const DevScene& D, cudaStream_t stream);

// Whether a material blocks shadow rays (shadowOccluded, PathTrace.metal:
// 4230-4241), and the opacity bits of a table's first 32 materials.
bool materialBlocksShadow(const dk_material& m);
uint32_t opaqueMask(const dk_material* mats, uint32_t count);

// A wave of `capPaths` paths, `pixelCap` AOV-record pixels and `jobCap` jobs.
int allocWave(Arena& arena, Wave& W, uint64_t capPaths, uint32_t pixelCap, uint32_t jobCap);
int allocAccum(Arena& arena, Accum& A, size_t pixels);
int clearAccum(const Accum& A, size_t pixels, cudaStream_t st);

// DevParams of a render from its settings (RenderSession.swift:908-947).
void fillParams(DevParams& P, const dk_settings& st);

struct Grids {
    int gen, extend, shade, shadow, final;
    int extend8, shadow8;  // the traversal kernels over the 8-wide tree
    int volume;            // the distance-volume pass (persistent: its resident blocks)
};
Grids kernelGrids();

// Launches one wave whose job table is already on the device: generation,
// `maxBounces` bounces (extend, shade, shadow + resolve), the denoiser AOV
// ray when `anyDenoiser`, finalize.  `mark(kind)` runs before each stage
// (0 other, 1 extend, 2 shade, 3 shadow) and once more at the end (0).
int launchWave(const DevScene& S, const Wave& W, uint32_t maxBounces, bool anyDenoiser, const Grids& g,
               cudaStream_t st, const std::function<int(int)>& mark, uint64_t& launches);

}  // namespace dk
