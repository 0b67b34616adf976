// Serving loop of the C ABI (dk_server_* in include/denrim_cuda.h).
//
// Resident scenes, many jobs.  The scene given at create is scene 0;
// dk_server_add_scene makes more resident (BVHs, textures, lights and the HDRI
// table stay on the device), each with its own wavefront and stream.  Every
// step packs, per scene, the paths of the oldest admitted jobs of that scene
// into the scene's wavefront (each job contributes up to `samples_per_wave`
// whole frames), so small previews that could never fill the GPU alone run
// side by side with larger renders; the scenes' waves are issued on their own
// streams and overlap on the device.  Per job the server keeps a material
// table in a slot of its scene's material array and one device block (from a
// private stream-ordered pool) with the job's Kahan accumulation buffers and
// AOV planes; admission is first-in first-out while those blocks fit the HBM
// budget.  Paths depend only on (pixel, sample, frame seed, the job's
// materials and settings) and every pixel accumulates its samples in order,
// so a job renders the same bits alone or in a mix, whatever the other
// scenes do.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>

#include "dk_host.h"

namespace {

using dk::fail;

constexpr size_t kAlign = 256;
inline size_t alignUp(size_t v) { return (v + kAlign - 1) & ~(kAlign - 1); }

// Bytes of one job's device block: Kahan sum + compensation, FP64 resolve,
// sample counts and six AOV planes per pixel.
size_t jobBlockBytes(size_t pixels) {
    return alignUp(pixels * sizeof(float4)) * 2 + alignUp(pixels * sizeof(dk::D4)) + alignUp(pixels * sizeof(uint32_t)) +
           alignUp(6 * pixels * sizeof(float4));
}

struct Job {
    uint64_t id = 0;
    uint32_t scene = 0;  // index into Server::scenes
    dk_settings settings;
    uint32_t samples = 0, samplesDone = 0, waves = 0, state = DK_JOB_QUEUED;
    std::vector<dk_material> materials;
    uint32_t slot = 0;  // material slot of its scene: S.mats[(1 + slot) * M, (2 + slot) * M)
    uint32_t opaqueMask = 0;
    dk::Accum A{};
    void* block = nullptr;
    size_t bytes = 0;
    double submitMs = 0, admitMs = 0, finishMs = 0;
};

// One resident scene: its device arrays (material array with one table per
// material slot), its wavefront and the stream its waves and admissions run on.
struct SceneSlot {
    dk::Arena arena;
    dk::DevScene scene;
    dk::Wave wave;
    cudaStream_t stream = nullptr;
    cudaEvent_t evBegin = nullptr, evEnd = nullptr;
    uint32_t matCount = 0;            // M: entries of the scene's (and its jobs') material table
    std::vector<dk_material> baseMaterials;
    std::vector<uint32_t> freeSlots;  // material slots (guarded by Server::mu)
};

struct Server {
    dk_server_config cfg;
    dk::Grids grids;
    std::vector<std::unique_ptr<SceneSlot>> scenes;  // appended under stepMu + mu; never removed
    cudaStream_t ioStream = nullptr;  // readback and release of finished jobs
    cudaMemPool_t pool = nullptr;
    float4* staging = nullptr;        // readback staging (ioStream), grown on demand
    size_t stagingPixels = 0;
    cudaEvent_t copyDone = nullptr;   // orders dk_server_copy_output before the caller's stream

    std::mutex mu;                    // jobs, queues, budget, stats
    std::condition_variable cv;
    std::mutex stepMu;                // one wave at a time
    std::mutex ioMu;                  // ioStream and staging
    std::deque<uint64_t> pending;
    std::vector<uint64_t> running;    // admission order
    std::unordered_map<uint64_t, std::unique_ptr<Job>> jobs;
    uint64_t nextId = 1;
    uint64_t budgetUsed = 0, budgetPeak = 0;
    uint64_t submitted = 0, done = 0, waves = 0, paths = 0, launches = 0;
    double busyMs = 0, jobsInWaveSum = 0, jobsInWaveMax = 0;
    std::thread worker;
    bool workerOn = false, stopFlag = false;
    int workerError = DK_OK;
    std::string workerMessage;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double nowMs() const {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    }
};

Server* asServer(dk_server* s) { return reinterpret_cast<Server*>(s); }

void destroyServer(Server* s) {
    if (!s) return;
    for (auto& sc : s->scenes)
        if (sc->stream) cudaStreamSynchronize(sc->stream);
    if (s->ioStream) cudaStreamSynchronize(s->ioStream);
    for (auto& kv : s->jobs)
        if (kv.second->block && s->ioStream) cudaFreeAsync(kv.second->block, s->ioStream);
    if (s->ioStream) cudaStreamSynchronize(s->ioStream);
    if (s->staging) cudaFree(s->staging);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    for (auto& sc : s->scenes) {
        sc->arena.release();
        if (sc->evBegin) cudaEventDestroy(sc->evBegin);
        if (sc->evEnd) cudaEventDestroy(sc->evEnd);
        if (sc->stream) cudaStreamDestroy(sc->stream);
    }
    if (s->copyDone) cudaEventDestroy(s->copyDone);
    if (s->ioStream) cudaStreamDestroy(s->ioStream);
    delete s;
}

// Uploads `sc` as a resident scene with its own wavefront and stream.
int makeSceneSlot(Server* s, const dk_scene* sc, std::unique_ptr<SceneSlot>& out) {
    int rc = dk::validateScene(sc);
    if (rc != DK_OK) return rc;
    auto slot = std::make_unique<SceneSlot>();
    SceneSlot& S = *slot;
    struct Cleanup {  // a failed upload releases what it made
        std::unique_ptr<SceneSlot>& p;
        bool keep = false;
        ~Cleanup() {
            if (keep || !p) return;
            p->arena.release();
            if (p->evBegin) cudaEventDestroy(p->evBegin);
            if (p->evEnd) cudaEventDestroy(p->evEnd);
            if (p->stream) cudaStreamDestroy(p->stream);
        }
    } cleanup{slot};
    DK_CUDA(cudaStreamCreateWithFlags(&S.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    DK_CUDA(cudaEventCreate(&S.evBegin), "cudaEventCreate");
    DK_CUDA(cudaEventCreate(&S.evEnd), "cudaEventCreate");
    S.matCount = sc->material_count;
    S.baseMaterials.assign(sc->materials, sc->materials + sc->material_count);
    const uint32_t slots = s->cfg.max_resident_jobs;
    rc = dk::uploadScene(S.arena, sc, S.scene,
                         (uint32_t)std::min<uint64_t>((uint64_t)(slots + 1) * S.matCount, 0xffffffffull));
    if (rc != DK_OK) return rc;
    S.scene.all_shadow_opaque = 0;  // job tables may make materials cut-out or transmissive
    for (uint32_t k = slots; k > 0; --k) S.freeSlots.push_back(k - 1);
    rc = dk::allocWave(S.arena, S.wave, s->cfg.wave_paths, s->cfg.wave_paths, s->cfg.max_jobs_per_wave);
    if (rc != DK_OK) return rc;
    cleanup.keep = true;
    out = std::move(slot);
    return DK_OK;
}

bool sameEmission(const dk_material& a, const dk_material& b) {
    return std::memcmp(&a.emission, &b.emission, 3 * sizeof(float)) == 0;
}

// Admits queued jobs in arrival order while their blocks fit the budget and a
// material slot is free.  Called with `mu` held.
int admitLocked(Server* s) {
    while (!s->pending.empty()) {
        Job& j = *s->jobs[s->pending.front()];
        SceneSlot& S = *s->scenes[j.scene];
        size_t pixels = (size_t)j.settings.width * j.settings.height;
        size_t bytes = jobBlockBytes(pixels);
        if (s->budgetUsed + bytes > s->cfg.hbm_budget_bytes || S.freeSlots.empty() ||
            s->running.size() >= s->cfg.max_resident_jobs)
            break;
        void* block = nullptr;
        DK_CUDA(cudaMallocFromPoolAsync(&block, bytes, s->pool, S.stream), "job buffers");
        char* p = static_cast<char*>(block);
        j.A.sum = reinterpret_cast<float4*>(p);
        p += alignUp(pixels * sizeof(float4));
        j.A.comp = reinterpret_cast<float4*>(p);
        p += alignUp(pixels * sizeof(float4));
        j.A.resolved = reinterpret_cast<dk::D4*>(p);
        p += alignUp(pixels * sizeof(dk::D4));
        j.A.count = reinterpret_cast<uint32_t*>(p);
        p += alignUp(pixels * sizeof(uint32_t));
        j.A.aov = reinterpret_cast<float4*>(p);
        DK_CUDA(cudaMemsetAsync(block, 0, bytes, S.stream), "job buffers");
        j.slot = S.freeSlots.back();
        S.freeSlots.pop_back();
        dk_material* dst = const_cast<dk_material*>(S.scene.mats) + (size_t)(1 + j.slot) * S.matCount;
        // Pageable source: staged before the call returns.
        DK_CUDA(cudaMemcpyAsync(dst, j.materials.data(), S.matCount * sizeof(dk_material), cudaMemcpyHostToDevice,
                                S.stream),
                "job materials");
        j.block = block;
        j.bytes = bytes;
        j.state = DK_JOB_RUNNING;
        j.admitMs = s->nowMs();
        s->budgetUsed += bytes;
        s->budgetPeak = std::max(s->budgetPeak, s->budgetUsed);
        s->running.push_back(j.id);
        s->pending.pop_front();
    }
    return DK_OK;
}

bool hasWorkLocked(Server* s) {
    for (uint64_t id : s->running)
        if (s->jobs[id]->state == DK_JOB_RUNNING) return true;
    if (s->pending.empty()) return false;
    const Job& j = *s->jobs.at(s->pending.front());
    size_t bytes = jobBlockBytes((size_t)j.settings.width * j.settings.height);
    return s->budgetUsed + bytes <= s->cfg.hbm_budget_bytes && !s->scenes[j.scene]->freeSlots.empty() &&
           s->running.size() < s->cfg.max_resident_jobs;
}

// Admission, one packed wave per scene with work (the scenes' waves overlap
// on their streams), completion.
int stepServer(Server* s, uint32_t* outJobs) {
    std::lock_guard<std::mutex> stepLock(s->stepMu);
    if (outJobs) *outJobs = 0;
    struct Plan {
        std::vector<dk::DevJob> table;
        std::vector<Job*> members;
        std::vector<uint32_t> counts;
        uint32_t maxBounces = 1;
        bool anyDenoiser = false;
    };
    std::vector<Plan> plans;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        int rc = admitLocked(s);
        if (rc != DK_OK) return rc;
        plans.resize(s->scenes.size());
        // Wave order per scene: its oldest running job first (it always
        // progresses), then the others by remaining paths, fewest first
        // (policy 1), or in admission order (policy 0).
        std::vector<std::vector<uint64_t>> order(s->scenes.size());
        for (uint64_t id : s->running) {
            const Job& j = *s->jobs[id];
            if (j.state == DK_JOB_RUNNING) order[j.scene].push_back(id);
        }
        for (size_t si = 0; si < s->scenes.size(); ++si) {
            std::vector<uint64_t>& ord = order[si];
            if (s->cfg.policy == 1 && ord.size() > 2) {
                auto remaining = [&](uint64_t id) {
                    const Job& j = *s->jobs[id];
                    return (uint64_t)(j.samples - j.samplesDone) * j.settings.width * j.settings.height;
                };
                std::stable_sort(ord.begin() + 1, ord.end(),
                                 [&](uint64_t x, uint64_t y) { return remaining(x) < remaining(y); });
            }
            const SceneSlot& S = *s->scenes[si];
            Plan& pl = plans[si];
            uint64_t used = 0, pix = 0;
            const uint64_t cap = S.wave.cap;
            for (uint64_t id : ord) {
                Job& j = *s->jobs[id];
                if (pl.table.size() >= s->cfg.max_jobs_per_wave) break;
                uint64_t pixels = (uint64_t)j.settings.width * j.settings.height;
                uint64_t room = (cap - used) / pixels;
                uint32_t nb = (uint32_t)std::min<uint64_t>({(uint64_t)(j.samples - j.samplesDone),
                                                             (uint64_t)s->cfg.samples_per_wave, room});
                if (nb == 0) continue;  // no room for a frame of this job; a smaller one may still fit
                dk::DevJob dj;
                std::memset(&dj, 0, sizeof(dj));
                dk::fillParams(dj.P, j.settings);
                dj.P.sample_begin = j.samplesDone;
                dj.P.samples_in_batch = nb;
                dj.P.path_count = (uint32_t)(nb * pixels);
                dj.A = j.A;
                dj.path_begin = (uint32_t)used;
                dj.pixel_begin = (uint32_t)pix;
                dj.mat_base = (1 + j.slot) * S.matCount;
                dj.mat_count = S.matCount;
                dj.opaque_mask = j.opaqueMask;
                pl.table.push_back(dj);
                pl.members.push_back(&j);
                pl.counts.push_back(nb);
                used += nb * pixels;
                pix += pixels;
                pl.maxBounces = std::max(pl.maxBounces, dj.P.max_bounces);
                pl.anyDenoiser = pl.anyDenoiser || dj.P.denoiser != 0;
            }
        }
    }
    uint64_t launches = 0, paths = 0;
    uint32_t jobsInStep = 0, wavesInStep = 0;
    int first = -1;
    for (size_t si = 0; si < plans.size(); ++si) {
        Plan& pl = plans[si];
        if (pl.table.empty()) continue;
        SceneSlot& S = *s->scenes[si];
        cudaStream_t q = S.stream;
        DK_CUDA(cudaMemcpyAsync(const_cast<dk::DevJob*>(S.wave.jobs), pl.table.data(),
                                pl.table.size() * sizeof(dk::DevJob), cudaMemcpyHostToDevice, q),
                "job table upload");
        dk::Wave W = S.wave;
        W.job_count = (uint32_t)pl.table.size();
        W.path_count = pl.table.back().path_begin + pl.table.back().P.path_count;
        W.pixel_count = pl.table.back().pixel_begin + pl.table.back().P.tile_w * pl.table.back().P.tile_h;
        DK_CUDA(cudaEventRecord(S.evBegin, q), "cudaEventRecord");
        auto mark = [](int) { return (int)DK_OK; };
        uint64_t l = 0;
        int rc = dk::launchWave(S.scene, W, pl.maxBounces, pl.anyDenoiser, s->grids, q, mark, l);
        if (rc != DK_OK) return rc;
        DK_CUDA(cudaEventRecord(S.evEnd, q), "cudaEventRecord");
        launches += l;
        paths += W.path_count;
        jobsInStep += W.job_count;
        wavesInStep += 1;
        if (first < 0) first = (int)si;
    }
    if (first < 0) return DK_OK;
    // Busy time of the step: from the first wave's start to the last end.
    float ms = 0;
    for (size_t si = 0; si < plans.size(); ++si) {
        if (plans[si].table.empty()) continue;
        DK_CUDA(cudaEventSynchronize(s->scenes[si]->evEnd), "wave");
        float e = 0;
        DK_CUDA(cudaEventElapsedTime(&e, s->scenes[first]->evBegin, s->scenes[si]->evEnd), "cudaEventElapsedTime");
        ms = std::max(ms, e);
    }
    {
        std::lock_guard<std::mutex> lk(s->mu);
        double now = s->nowMs();
        for (const Plan& pl : plans)
            for (size_t k = 0; k < pl.members.size(); ++k) {
                Job& j = *pl.members[k];
                j.samplesDone += pl.counts[k];
                j.waves += 1;
                if (j.samplesDone >= j.samples) {
                    j.state = DK_JOB_DONE;
                    j.finishMs = now;
                    s->done += 1;
                }
            }
        s->waves += wavesInStep;
        s->paths += paths;
        s->launches += launches;
        s->busyMs += ms;
        s->jobsInWaveSum += (double)jobsInStep;
        s->jobsInWaveMax = std::max(s->jobsInWaveMax, (double)jobsInStep / wavesInStep);
    }
    s->cv.notify_all();
    if (outJobs) *outJobs = jobsInStep;
    return DK_OK;
}

void workerLoop(Server* s) {
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv.wait(lk, [&] { return s->stopFlag || hasWorkLocked(s); });
            if (s->stopFlag) return;
        }
        int rc = stepServer(s, nullptr);
        if (rc != DK_OK) {
            std::lock_guard<std::mutex> lk(s->mu);
            s->workerError = rc;
            s->workerMessage = dk_last_error_message();
            s->stopFlag = true;
            s->cv.notify_all();
            return;
        }
    }
}

// The scene a job names, or null (under mu: the list only grows).
const SceneSlot* jobScene(Server* s, uint32_t index) {
    std::lock_guard<std::mutex> lk(s->mu);
    return index < s->scenes.size() ? s->scenes[index].get() : nullptr;
}

int validateJob(Server* s, const dk_job_desc* jd) {
    const SceneSlot* S = jobScene(s, jd->scene);
    if (!S) return fail(DK_ERROR_INVALID_ARGUMENT, "a job names a scene the server does not hold");
    const dk_settings& st = jd->settings;
    if (st.width == 0 || st.height == 0)
        return fail(DK_ERROR_INVALID_SCENE, "Invalid render scene: Render dimensions must be positive.");
    if (st.quality != DK_QUALITY_FINAL)
        return fail(DK_ERROR_INVALID_ARGUMENT, "only RenderQuality.final (the path tracer) is implemented");
    if (jd->samples == 0) return fail(DK_ERROR_INVALID_ARGUMENT, "a job must render at least one sample");
    uint64_t pixels = (uint64_t)st.width * st.height;
    if (pixels > S->wave.cap) return fail(DK_ERROR_INVALID_ARGUMENT, "one frame of the job exceeds the wave capacity");
    if (jobBlockBytes(pixels) > s->cfg.hbm_budget_bytes)
        return fail(DK_ERROR_OUT_OF_MEMORY, "the job's buffers exceed the server's HBM budget");
    if (jd->material_count != S->matCount || !jd->materials)
        return fail(DK_ERROR_INVALID_ARGUMENT, "a job's material table must have the scene's material count");
    for (uint32_t i = 0; i < S->matCount; ++i) {
        const dk_material& m = jd->materials[i];
        const dk_material& b = S->baseMaterials[i];
        if (!sameEmission(m, b))
            return fail(DK_ERROR_INVALID_ARGUMENT, "a job may not change a material's emission (the light list is shared)");
        if (i >= 32 && dk::materialBlocksShadow(m) != dk::materialBlocksShadow(b))
            return fail(DK_ERROR_INVALID_ARGUMENT,
                        "a job may not change whether material IDs from 32 up block shadow rays");
        float texB = m.parameters.z, texN = m.parameters.w;
        if (texB < 0.0f || texN < 0.0f || texB > (float)S->scene.texdesc_count || texN > (float)S->scene.texdesc_count)
            return fail(DK_ERROR_INVALID_ARGUMENT, "a job material references a texture the scene does not have");
    }
    return DK_OK;
}

}  // namespace

extern "C" {

int dk_server_create(const dk_scene* sc, const dk_server_config* config, dk_server** out) {
    if (!sc || !out) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_server_create: null argument");
    *out = nullptr;
    int rc = dk::validateScene(sc);
    if (rc != DK_OK) return rc;
    rc = dk::ensureDevice();
    if (rc != DK_OK) return rc;
    Server* s = new Server();
    std::memset(&s->cfg, 0, sizeof(s->cfg));
    if (config) s->cfg = *config;
    if (s->cfg.hbm_budget_bytes == 0) s->cfg.hbm_budget_bytes = 64ull << 30;
    if (s->cfg.wave_paths == 0) s->cfg.wave_paths = 1u << 24;
    if (s->cfg.max_jobs_per_wave == 0) s->cfg.max_jobs_per_wave = 512;
    if (s->cfg.max_resident_jobs == 0) s->cfg.max_resident_jobs = 4096;
    if (s->cfg.samples_per_wave == 0) s->cfg.samples_per_wave = 64;
    if (s->cfg.policy > 1) {
        destroyServer(s);
        return fail(DK_ERROR_INVALID_ARGUMENT, "dk_server_config.policy must be 0 or 1");
    }
    s->cfg.wave_paths = std::min<uint32_t>(s->cfg.wave_paths, 1u << 29);  // path indices fit 29 bits
#define TRY_CUDA(x, what)                                                                          \
    do {                                                                                           \
        cudaError_t _e = (x);                                                                      \
        if (_e != cudaSuccess) {                                                                   \
            destroyServer(s);                                                                      \
            return fail(DK_ERROR_COMMAND_FAILED, std::string(what) + ": " + cudaGetErrorString(_e)); \
        }                                                                                          \
    } while (0)
    TRY_CUDA(cudaStreamCreateWithFlags(&s->ioStream, cudaStreamNonBlocking), "cudaStreamCreate");
    int device = 0;
    TRY_CUDA(cudaGetDevice(&device), "cudaGetDevice");
    cudaMemPoolProps props;
    std::memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    TRY_CUDA(cudaMemPoolCreate(&s->pool, &props), "cudaMemPoolCreate");
    uint64_t keep = ~0ull;  // keep freed job blocks in the pool for the next admissions
    TRY_CUDA(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep), "cudaMemPoolSetAttribute");
#undef TRY_CUDA
    std::unique_ptr<SceneSlot> first;
    rc = makeSceneSlot(s, sc, first);
    if (rc != DK_OK) {
        destroyServer(s);
        return rc;
    }
    s->scenes.push_back(std::move(first));
    s->grids = dk::kernelGrids();
    *out = reinterpret_cast<dk_server*>(s);
    return DK_OK;
}

int dk_server_add_scene(dk_server* server, const dk_scene* sc, uint32_t* outScene) {
    Server* s = asServer(server);
    if (!s || !sc || !outScene) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_server_add_scene: null argument");
    std::unique_ptr<SceneSlot> slot;
    int rc = makeSceneSlot(s, sc, slot);
    if (rc != DK_OK) return rc;
    std::lock_guard<std::mutex> stepLock(s->stepMu);  // no wave reads the list meanwhile
    std::lock_guard<std::mutex> lk(s->mu);
    *outScene = (uint32_t)s->scenes.size();
    s->scenes.push_back(std::move(slot));
    return DK_OK;
}

int dk_server_submit(dk_server* server, const dk_job_desc* jd, uint64_t* outId) {
    Server* s = asServer(server);
    if (!s || !jd || !outId) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_server_submit: null argument");
    int rc = validateJob(s, jd);
    if (rc != DK_OK) return rc;
    auto j = std::make_unique<Job>();
    j->scene = jd->scene;
    j->settings = jd->settings;
    if (j->settings.max_bounces < 1) j->settings.max_bounces = 1;
    j->samples = jd->samples;
    j->materials.assign(jd->materials, jd->materials + jd->material_count);
    j->opaqueMask = dk::opaqueMask(j->materials.data(), jd->material_count);
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->workerError != DK_OK) return fail(s->workerError, "server stopped: " + s->workerMessage);
        j->id = s->nextId++;
        j->submitMs = s->nowMs();
        *outId = j->id;
        s->pending.push_back(j->id);
        s->jobs.emplace(j->id, std::move(j));
        s->submitted += 1;
    }
    s->cv.notify_all();
    return DK_OK;
}

int dk_server_step(dk_server* server, uint32_t* outJobs) {
    Server* s = asServer(server);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "server is null");
    return stepServer(s, outJobs);
}

int dk_server_start(dk_server* server) {
    Server* s = asServer(server);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "server is null");
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->workerOn) return DK_OK;
    s->stopFlag = false;
    s->workerError = DK_OK;
    s->workerOn = true;
    s->worker = std::thread(workerLoop, s);
    return DK_OK;
}

int dk_server_stop(dk_server* server) {
    Server* s = asServer(server);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "server is null");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (!s->workerOn) return DK_OK;
        s->stopFlag = true;
    }
    s->cv.notify_all();
    s->worker.join();
    std::lock_guard<std::mutex> lk(s->mu);
    s->workerOn = false;
    if (s->workerError != DK_OK) return fail(s->workerError, "server stopped: " + s->workerMessage);
    return DK_OK;
}

int dk_server_wait(dk_server* server, uint64_t id, uint32_t timeoutMs) {
    Server* s = asServer(server);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "server is null");
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return fail(DK_ERROR_INVALID_ARGUMENT, "unknown job id");
    Job* j = it->second.get();
    bool ok = s->cv.wait_for(lk, std::chrono::milliseconds(timeoutMs),
                             [&] { return j->state >= DK_JOB_DONE || s->workerError != DK_OK; });
    if (s->workerError != DK_OK) return fail(s->workerError, "server stopped: " + s->workerMessage);
    if (!ok) return fail(DK_ERROR_DEVICE_TIMEOUT, "job not finished within the timeout");
    return DK_OK;
}

int dk_server_job_status(dk_server* server, uint64_t id, dk_job_status* out) {
    Server* s = asServer(server);
    if (!s || !out) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->jobs.find(id);
    if (it == s->jobs.end()) return fail(DK_ERROR_INVALID_ARGUMENT, "unknown job id");
    const Job& j = *it->second;
    out->job_id = j.id;
    out->state = j.state;
    out->samples_done = j.samplesDone;
    out->samples = j.samples;
    out->waves = j.waves;
    out->submit_ms = j.submitMs;
    out->admit_ms = j.admitMs;
    out->finish_ms = j.finishMs;
    return DK_OK;
}

namespace {

// A finished job's output plane on the device (the beauty resolved into the
// staging buffer on the I/O stream, or an AOV plane).  Called with ioMu held.
int jobPlane(Server* s, uint64_t id, int output, size_t pixelCount, const float4** src) {
    if (output < DK_OUTPUT_BEAUTY || output > DK_OUTPUT_MOTION_VECTOR)
        return fail(DK_ERROR_INVALID_ARGUMENT, "unknown output kind");
    dk::Accum A;
    size_t pixels;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(id);
        if (it == s->jobs.end()) return fail(DK_ERROR_INVALID_ARGUMENT, "unknown job id");
        const Job& j = *it->second;
        if (j.state != DK_JOB_DONE) return fail(DK_ERROR_INVALID_ARGUMENT, "the job has not finished (or was released)");
        A = j.A;
        pixels = (size_t)j.settings.width * j.settings.height;
    }
    if (pixelCount != pixels) return fail(DK_ERROR_INVALID_ARGUMENT, "pixel_count must equal width*height");
    // The job's last wave was synchronized before DONE was set, and no later
    // wave touches its buffers: reading them needs no ordering with the wave
    // stream.
    if (output == DK_OUTPUT_BEAUTY) {
        if (s->stagingPixels < pixels) {
            if (s->staging) cudaFree(s->staging);
            s->staging = nullptr;
            s->stagingPixels = 0;
            DK_CUDA(cudaMalloc(&s->staging, pixels * sizeof(float4)), "readback staging");
            s->stagingPixels = pixels;
        }
        DK_CUDA(dk::launchResolveBeauty(A, (uint32_t)pixels, s->staging, s->grids.final, s->ioStream), "resolve launch");
        *src = s->staging;
    } else {
        *src = A.aov + (size_t)(output - 1) * pixels;
    }
    return DK_OK;
}

}  // namespace

int dk_server_read_output(dk_server* server, uint64_t id, int output, float* rgba, size_t pixelCount) {
    Server* s = asServer(server);
    if (!s || !rgba) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> io(s->ioMu);
    const float4* src = nullptr;
    int rc = jobPlane(s, id, output, pixelCount, &src);
    if (rc != DK_OK) return rc;
    DK_CUDA(cudaMemcpyAsync(rgba, src, pixelCount * sizeof(float4), cudaMemcpyDeviceToHost, s->ioStream), "readback");
    DK_CUDA(cudaStreamSynchronize(s->ioStream), "readback");
    return DK_OK;
}

int dk_server_copy_output(dk_server* server, uint64_t id, int output, void* deviceRgba, size_t pixelCount,
                          void* stream) {
    return dk_server_copy_outputs(server, &id, 1, output, deviceRgba, pixelCount, 0, stream);
}

int dk_server_copy_outputs(dk_server* server, const uint64_t* ids, size_t count, int output, void* deviceRgba,
                           size_t pixelCount, size_t strideBytes, void* stream) {
    Server* s = asServer(server);
    if (!s || !ids || !deviceRgba) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    if (strideBytes == 0) strideBytes = pixelCount * sizeof(float4);
    if (reinterpret_cast<uintptr_t>(deviceRgba) % 16u || strideBytes % 16u)
        return fail(DK_ERROR_INVALID_ARGUMENT, "device_rgba and the stride must be 16-byte aligned");
    if (count > 1 && strideBytes < pixelCount * sizeof(float4))
        return fail(DK_ERROR_INVALID_ARGUMENT, "the stride is smaller than one image");
    std::lock_guard<std::mutex> io(s->ioMu);
    for (size_t i = 0; i < count; ++i) {
        const float4* src = nullptr;
        int rc = jobPlane(s, ids[i], output, pixelCount, &src);
        if (rc != DK_OK) return rc;
        DK_CUDA(cudaMemcpyAsync(static_cast<char*>(deviceRgba) + i * strideBytes, src, pixelCount * sizeof(float4),
                                cudaMemcpyDeviceToDevice, s->ioStream),
                "output copy");
    }
    if (!stream) {
        DK_CUDA(cudaStreamSynchronize(s->ioStream), "output copy");
        return DK_OK;
    }
    if (!s->copyDone) DK_CUDA(cudaEventCreateWithFlags(&s->copyDone, cudaEventDisableTiming), "cudaEventCreate");
    DK_CUDA(cudaEventRecord(s->copyDone, s->ioStream), "cudaEventRecord");
    DK_CUDA(cudaStreamWaitEvent(static_cast<cudaStream_t>(stream), s->copyDone, 0), "cudaStreamWaitEvent");
    return DK_OK;
}

int dk_server_release(dk_server* server, uint64_t id) {
    Server* s = asServer(server);
    if (!s) return fail(DK_ERROR_INVALID_ARGUMENT, "server is null");
    {
        std::lock_guard<std::mutex> io(s->ioMu);
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->jobs.find(id);
        if (it == s->jobs.end()) return fail(DK_ERROR_INVALID_ARGUMENT, "unknown job id");
        Job& j = *it->second;
        if (j.state == DK_JOB_RELEASED) return DK_OK;
        if (j.state != DK_JOB_DONE) return fail(DK_ERROR_INVALID_ARGUMENT, "only finished jobs can be released");
        DK_CUDA(cudaFreeAsync(j.block, s->ioStream), "release job buffers");
        j.block = nullptr;
        s->budgetUsed -= j.bytes;
        s->scenes[j.scene]->freeSlots.push_back(j.slot);
        s->running.erase(std::find(s->running.begin(), s->running.end(), j.id));
        j.state = DK_JOB_RELEASED;
        j.materials.clear();
        j.materials.shrink_to_fit();
    }
    s->cv.notify_all();
    return DK_OK;
}

int dk_server_get_stats(dk_server* server, dk_server_stats* out) {
    Server* s = asServer(server);
    if (!s || !out) return fail(DK_ERROR_INVALID_ARGUMENT, "null argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->jobs_submitted = s->submitted;
    out->jobs_done = s->done;
    out->jobs_queued = s->pending.size();
    uint64_t run = 0;
    for (uint64_t id : s->running)
        if (s->jobs[id]->state == DK_JOB_RUNNING) ++run;
    out->jobs_running = run;
    out->waves = s->waves;
    out->paths_traced = s->paths;
    out->kernel_launches = s->launches;
    out->budget_used_bytes = s->budgetUsed;
    out->budget_peak_bytes = s->budgetPeak;
    uint64_t sceneBytes = 0;
    for (const auto& sc : s->scenes) sceneBytes += sc->arena.bytes;
    out->device_bytes = sceneBytes + s->budgetUsed;
    out->busy_ms = s->busyMs;
    out->max_jobs_in_wave = s->jobsInWaveMax;
    out->mean_jobs_in_wave = s->waves ? s->jobsInWaveSum / (double)s->waves : 0.0;
    return DK_OK;
}

int dk_server_destroy(dk_server* server) {
    Server* s = asServer(server);
    if (!s) return DK_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stopFlag = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    destroyServer(s);
    return DK_OK;
}

}  // extern "C"
