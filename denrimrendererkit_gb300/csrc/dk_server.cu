// Serving loop of the C ABI (dk_server_* in include/denrim_cuda.h).
//
// One resident scene, many jobs.  Every wave packs the paths of the oldest
// admitted jobs into the shared wavefront (each job contributes up to
// `samples_per_wave` whole frames), so small previews that could never fill
// the GPU alone run side by side with larger renders.  Per job the server
// keeps a material table in a slot of the scene's material array and one
// device block (from a private stream-ordered pool) with the job's Kahan
// accumulation buffers and AOV planes; admission is first-in first-out while
// those blocks fit the HBM budget.  Paths depend only on (pixel, sample,
// frame seed, the job's materials and settings) and every pixel accumulates
// its samples in order, so a job renders the same bits alone or in a mix.
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
    dk_settings settings;
    uint32_t samples = 0, samplesDone = 0, waves = 0, state = DK_JOB_QUEUED;
    std::vector<dk_material> materials;
    uint32_t slot = 0;  // material slot: S.mats[(1 + slot) * M, (2 + slot) * M)
    uint32_t opaqueMask = 0;
    dk::Accum A{};
    void* block = nullptr;
    size_t bytes = 0;
    double submitMs = 0, admitMs = 0, finishMs = 0;
};

struct Server {
    dk_server_config cfg;
    dk::Arena arena;
    dk::DevScene scene;
    dk::Wave wave;
    dk::Grids grids;
    cudaStream_t stream = nullptr;    // waves, admission uploads
    cudaStream_t ioStream = nullptr;  // readback and release of finished jobs
    cudaMemPool_t pool = nullptr;
    cudaEvent_t evBegin = nullptr, evEnd = nullptr;
    float4* staging = nullptr;        // readback staging (ioStream), grown on demand
    size_t stagingPixels = 0;
    cudaEvent_t copyDone = nullptr;   // orders dk_server_copy_output before the caller's stream
    uint32_t matCount = 0;            // M: entries of the scene's (and every job's) material table
    std::vector<dk_material> baseMaterials;
    std::vector<uint32_t> freeSlots;

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
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->ioStream) cudaStreamSynchronize(s->ioStream);
    for (auto& kv : s->jobs)
        if (kv.second->block) cudaFreeAsync(kv.second->block, s->stream);
    if (s->stream) cudaStreamSynchronize(s->stream);
    if (s->staging) cudaFree(s->staging);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    s->arena.release();
    if (s->evBegin) cudaEventDestroy(s->evBegin);
    if (s->evEnd) cudaEventDestroy(s->evEnd);
    if (s->copyDone) cudaEventDestroy(s->copyDone);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->ioStream) cudaStreamDestroy(s->ioStream);
    delete s;
}

bool sameEmission(const dk_material& a, const dk_material& b) {
    return std::memcmp(&a.emission, &b.emission, 3 * sizeof(float)) == 0;
}

// Admits queued jobs in arrival order while their blocks fit the budget and a
// material slot is free.  Called with `mu` held.
int admitLocked(Server* s) {
    while (!s->pending.empty()) {
        Job& j = *s->jobs[s->pending.front()];
        size_t pixels = (size_t)j.settings.width * j.settings.height;
        size_t bytes = jobBlockBytes(pixels);
        if (s->budgetUsed + bytes > s->cfg.hbm_budget_bytes || s->freeSlots.empty() ||
            s->running.size() >= s->cfg.max_resident_jobs)
            break;
        void* block = nullptr;
        DK_CUDA(cudaMallocFromPoolAsync(&block, bytes, s->pool, s->stream), "job buffers");
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
        DK_CUDA(cudaMemsetAsync(block, 0, bytes, s->stream), "job buffers");
        j.slot = s->freeSlots.back();
        s->freeSlots.pop_back();
        dk_material* dst = const_cast<dk_material*>(s->scene.mats) + (size_t)(1 + j.slot) * s->matCount;
        // Pageable source: staged before the call returns.
        DK_CUDA(cudaMemcpyAsync(dst, j.materials.data(), s->matCount * sizeof(dk_material), cudaMemcpyHostToDevice,
                                s->stream),
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
    return s->budgetUsed + bytes <= s->cfg.hbm_budget_bytes && !s->freeSlots.empty() &&
           s->running.size() < s->cfg.max_resident_jobs;
}

// Admission, one packed wave, completion.
int stepServer(Server* s, uint32_t* outJobs) {
    std::lock_guard<std::mutex> stepLock(s->stepMu);
    if (outJobs) *outJobs = 0;
    std::vector<dk::DevJob> table;
    std::vector<Job*> members;
    std::vector<uint32_t> counts;
    uint32_t maxBounces = 1;
    bool anyDenoiser = false;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        int rc = admitLocked(s);
        if (rc != DK_OK) return rc;
        uint64_t used = 0, pix = 0;
        const uint64_t cap = s->wave.cap;
        // Wave order: the oldest running job first (it always progresses), then
        // the others by remaining paths, fewest first (policy 1), or in
        // admission order (policy 0).
        std::vector<uint64_t> order;
        for (uint64_t id : s->running)
            if (s->jobs[id]->state == DK_JOB_RUNNING) order.push_back(id);
        if (s->cfg.policy == 1 && order.size() > 2) {
            auto remaining = [&](uint64_t id) {
                const Job& j = *s->jobs[id];
                return (uint64_t)(j.samples - j.samplesDone) * j.settings.width * j.settings.height;
            };
            std::stable_sort(order.begin() + 1, order.end(),
                             [&](uint64_t x, uint64_t y) { return remaining(x) < remaining(y); });
        }
        for (uint64_t id : order) {
            Job& j = *s->jobs[id];
            if (table.size() >= s->cfg.max_jobs_per_wave) break;
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
            dj.mat_base = (1 + j.slot) * s->matCount;
            dj.mat_count = s->matCount;
            dj.opaque_mask = j.opaqueMask;
            table.push_back(dj);
            members.push_back(&j);
            counts.push_back(nb);
            used += nb * pixels;
            pix += pixels;
            maxBounces = std::max(maxBounces, dj.P.max_bounces);
            anyDenoiser = anyDenoiser || dj.P.denoiser != 0;
        }
    }
    if (table.empty()) return DK_OK;
    cudaStream_t q = s->stream;
    DK_CUDA(cudaMemcpyAsync(const_cast<dk::DevJob*>(s->wave.jobs), table.data(), table.size() * sizeof(dk::DevJob),
                            cudaMemcpyHostToDevice, q),
            "job table upload");
    dk::Wave W = s->wave;
    W.job_count = (uint32_t)table.size();
    W.path_count = table.back().path_begin + table.back().P.path_count;
    W.pixel_count = table.back().pixel_begin + table.back().P.tile_w * table.back().P.tile_h;
    DK_CUDA(cudaEventRecord(s->evBegin, q), "cudaEventRecord");
    uint64_t launches = 0;
    auto mark = [](int) { return (int)DK_OK; };
    int rc = dk::launchWave(s->scene, W, maxBounces, anyDenoiser, s->grids, q, mark, launches);
    if (rc != DK_OK) return rc;
    DK_CUDA(cudaEventRecord(s->evEnd, q), "cudaEventRecord");
    DK_CUDA(cudaEventSynchronize(s->evEnd), "wave");
    float ms = 0;
    DK_CUDA(cudaEventElapsedTime(&ms, s->evBegin, s->evEnd), "cudaEventElapsedTime");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        double now = s->nowMs();
        for (size_t k = 0; k < members.size(); ++k) {
            Job& j = *members[k];
            j.samplesDone += counts[k];
            j.waves += 1;
            if (j.samplesDone >= j.samples) {
                j.state = DK_JOB_DONE;
                j.finishMs = now;
                s->done += 1;
            }
        }
        s->waves += 1;
        s->paths += W.path_count;
        s->launches += launches;
        s->busyMs += ms;
        s->jobsInWaveSum += (double)table.size();
        s->jobsInWaveMax = std::max(s->jobsInWaveMax, (double)table.size());
    }
    s->cv.notify_all();
    if (outJobs) *outJobs = (uint32_t)table.size();
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

int validateJob(Server* s, const dk_job_desc* jd) {
    const dk_settings& st = jd->settings;
    if (st.width == 0 || st.height == 0)
        return fail(DK_ERROR_INVALID_SCENE, "Invalid render scene: Render dimensions must be positive.");
    if (st.quality != DK_QUALITY_FINAL)
        return fail(DK_ERROR_INVALID_ARGUMENT, "only RenderQuality.final (the path tracer) is implemented");
    if (jd->samples == 0) return fail(DK_ERROR_INVALID_ARGUMENT, "a job must render at least one sample");
    uint64_t pixels = (uint64_t)st.width * st.height;
    if (pixels > s->wave.cap) return fail(DK_ERROR_INVALID_ARGUMENT, "one frame of the job exceeds the wave capacity");
    if (jobBlockBytes(pixels) > s->cfg.hbm_budget_bytes)
        return fail(DK_ERROR_OUT_OF_MEMORY, "the job's buffers exceed the server's HBM budget");
    if (jd->material_count != s->matCount || !jd->materials)
        return fail(DK_ERROR_INVALID_ARGUMENT, "a job's material table must have the scene's material count");
    for (uint32_t i = 0; i < s->matCount; ++i) {
        const dk_material& m = jd->materials[i];
        const dk_material& b = s->baseMaterials[i];
        if (!sameEmission(m, b))
            return fail(DK_ERROR_INVALID_ARGUMENT, "a job may not change a material's emission (the light list is shared)");
        if (i >= 32 && dk::materialBlocksShadow(m) != dk::materialBlocksShadow(b))
            return fail(DK_ERROR_INVALID_ARGUMENT,
                        "a job may not change whether material IDs from 32 up block shadow rays");
        float texB = m.parameters.z, texN = m.parameters.w;
        if (texB < 0.0f || texN < 0.0f || texB > (float)s->scene.texdesc_count || texN > (float)s->scene.texdesc_count)
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
#define TRY(x)                  \
    do {                        \
        int _rc = (x);          \
        if (_rc != DK_OK) {     \
            destroyServer(s);   \
            return _rc;         \
        }                       \
    } while (0)
#define TRY_CUDA(x, what)                                                                          \
    do {                                                                                           \
        cudaError_t _e = (x);                                                                      \
        if (_e != cudaSuccess) {                                                                   \
            destroyServer(s);                                                                      \
            return fail(DK_ERROR_COMMAND_FAILED, std::string(what) + ": " + cudaGetErrorString(_e)); \
        }                                                                                          \
    } while (0)
    TRY_CUDA(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
    TRY_CUDA(cudaStreamCreateWithFlags(&s->ioStream, cudaStreamNonBlocking), "cudaStreamCreate");
    TRY_CUDA(cudaEventCreate(&s->evBegin), "cudaEventCreate");
    TRY_CUDA(cudaEventCreate(&s->evEnd), "cudaEventCreate");
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

    s->matCount = sc->material_count;
    s->baseMaterials.assign(sc->materials, sc->materials + sc->material_count);
    const uint32_t slots = s->cfg.max_resident_jobs;
    TRY(dk::uploadScene(s->arena, sc, s->scene, (uint32_t)std::min<uint64_t>((uint64_t)(slots + 1) * s->matCount,
                                                                             0xffffffffull)));
    s->scene.all_shadow_opaque = 0;  // job tables may make materials cut-out or transmissive
    for (uint32_t k = slots; k > 0; --k) s->freeSlots.push_back(k - 1);
    TRY(dk::allocWave(s->arena, s->wave, s->cfg.wave_paths, s->cfg.wave_paths, s->cfg.max_jobs_per_wave));
    s->grids = dk::kernelGrids();
#undef TRY
#undef TRY_CUDA
    *out = reinterpret_cast<dk_server*>(s);
    return DK_OK;
}

int dk_server_submit(dk_server* server, const dk_job_desc* jd, uint64_t* outId) {
    Server* s = asServer(server);
    if (!s || !jd || !outId) return fail(DK_ERROR_INVALID_ARGUMENT, "dk_server_submit: null argument");
    int rc = validateJob(s, jd);
    if (rc != DK_OK) return rc;
    auto j = std::make_unique<Job>();
    j->settings = jd->settings;
    if (j->settings.max_bounces < 1) j->settings.max_bounces = 1;
    j->samples = jd->samples;
    j->materials.assign(jd->materials, jd->materials + s->matCount);
    j->opaqueMask = dk::opaqueMask(j->materials.data(), s->matCount);
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
        s->freeSlots.push_back(j.slot);
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
    out->device_bytes = s->arena.bytes + s->budgetUsed;
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
