// Serving: step requests for many resident scenes, batched continuously.
//
// Submitters push {scene, steps, tag} into a lock-free ring (ring.h).  One
// worker thread owns everything else: per-scene FIFOs of requests, the ready
// order (scenes whose head request waits, in arrival order), residency under
// the device budget with least-recently-used spills to pinned host memory,
// and up to four waves in flight.  A wave takes every ready scene that is not
// already on the device (one request each) and launches, on the wave's own
// stream, the batched group kernel over all their island groups
// (batch.cu) -- each CTA running its request's steps back to back -- plus the
// one-scene path for scenes the batched kernel cannot take.  Completion of a
// wave is seen through its event; its requests go to the completion ring.  A
// scene is in at most one wave at a time, so its requests run in submission
// order and every result equals stepping that scene alone.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "groups_device.cuh"
#include "ring.h"

namespace bepugpu {

namespace {

double NowUs() {
    using namespace std::chrono;
    return (double)duration_cast<nanoseconds>(steady_clock::now().time_since_epoch()).count() * 1e-3;
}

struct ServeRequest {
    int32_t scene;
    uint32_t steps;
    uint64_t tag;
    double submitUs;
};

}  // namespace

struct Server {
    Context* ctx = nullptr;
    Context sink;  // the worker's error sink: the caller's context is not written from the worker
    bepugpu_server_config cfg{};
    StepParams p{};
    Ring<ServeRequest> submitQ;
    Ring<bepugpu_completion> doneQ;
    std::thread worker;
    std::atomic<bool> stop{false};
    std::atomic<uint64_t> submitted{0}, completed{0};
    std::mutex wakeMu;
    std::condition_variable wake;
    std::string lastError;
    std::mutex errMu;

    struct Slot {
        Scene* s = nullptr;
        std::deque<ServeRequest> pending;
        bool inFlight = false;
        bool queued = false;  // in the ready order
        uint64_t lastUse = 0;
        bool live = true;
    };
    std::mutex regMu;  // guards slots / slotOf between the worker and add / release
    std::vector<Slot> slots;
    std::unordered_map<int32_t, int> slotOf;
    std::deque<int> ready;
    uint64_t useClock = 0;

    std::vector<SceneView> viewsHost;
    SceneView* viewsDev = nullptr;
    size_t viewsCap = 0;
    std::vector<int> dirtyViews;

    struct Wave {
        cudaStream_t stream = nullptr;
        cudaEvent_t done = nullptr;
        int4* workDev = nullptr;
        int4* workHost = nullptr;  // pinned
        size_t workCap = 0;
        std::vector<int> slotIds;
        std::vector<ServeRequest> reqs;
        bool busy = false;
        double startUs = 0;
        uint32_t id = 0;
    };
    std::vector<Wave> waves;
    uint32_t waveCounter = 0;

    // stats (worker-written, read under regMu)
    uint64_t statWaves = 0, statWaveScenes = 0, statLaunches = 0, statSpills = 0, statRestores = 0;
    uint64_t statRoomWaits = 0, statRestoreFailures = 0;
    uint64_t residentBytes = 0, peakResident = 0, spilledBytes = 0;

    Server(size_t cap) : submitQ(cap), doneQ(cap) {}

    void SetError(const std::string& e) {
        std::lock_guard<std::mutex> g(errMu);
        lastError = e;
    }

    void Complete(const ServeRequest& r, int32_t status, uint32_t wave, double startUs) {
        bepugpu_completion c;
        c.tag = r.tag;
        c.scene = r.scene;
        c.status = status;
        c.steps = r.steps;
        c.wave = wave;
        c.submit_us = r.submitUs;
        c.start_us = startUs;
        c.done_us = NowUs();
        // The completion ring has the submit ring's capacity; a full ring means
        // nobody polls: wait for room rather than drop a result.
        while (!doneQ.Push(c)) {
            if (stop.load()) return;
            std::this_thread::yield();
        }
        completed.fetch_add(1, std::memory_order_release);
    }

    // Spill least recently used idle scenes until `need` more bytes fit.
    bool MakeRoom(size_t need) {
        while (residentBytes + need > cfg.device_budget_bytes) {
            int victim = -1;
            for (int i = 0; i < (int)slots.size(); i++) {
                const Slot& v = slots[i];
                if (!v.live || !v.s->arena || v.inFlight || !v.pending.empty()) continue;
                if (victim < 0 || v.lastUse < slots[victim].lastUse) victim = i;
            }
            if (victim < 0) return false;
            Scene* s = slots[victim].s;
            size_t bytes = s->DeviceBytes();
            if (s->Spill(&sink) != BEPUGPU_OK) {
                SetError(sink.lastError);
                return false;
            }
            residentBytes -= bytes;
            spilledBytes += bytes;
            statSpills++;
        }
        return true;
    }

    void EnsureViewCapacity() {
        if (viewsCap >= viewsHost.size()) return;
        size_t want = std::max<size_t>(viewsHost.size(), viewsCap * 2);
        SceneView* d = nullptr;
        if (cudaMalloc(&d, sizeof(SceneView) * want) != cudaSuccess) return;
        if (viewsDev) {
            cudaDeviceSynchronize();  // no wave reads the old table any more
            cudaFree(viewsDev);
        }
        viewsDev = d;
        viewsCap = want;
        dirtyViews.clear();
        for (int i = 0; i < (int)viewsHost.size(); i++) dirtyViews.push_back(i);
    }

    bool FinishWaves() {
        bool any = false;
        for (Wave& w : waves) {
            if (!w.busy) continue;
            cudaError_t e = cudaEventQuery(w.done);
            if (e == cudaErrorNotReady) continue;
            int32_t status = e == cudaSuccess ? BEPUGPU_OK : BEPUGPU_CUDA_ERROR;
            if (e != cudaSuccess) SetError(std::string("wave: ") + cudaGetErrorString(e));
            std::lock_guard<std::mutex> g(regMu);
            for (size_t k = 0; k < w.slotIds.size(); k++) {
                Slot& sl = slots[w.slotIds[k]];
                sl.inFlight = false;
                sl.lastUse = ++useClock;
                sl.s->asyncPending = false;
                if (!sl.pending.empty() && !sl.queued) {
                    sl.queued = true;
                    ready.push_back(w.slotIds[k]);
                }
                Complete(w.reqs[k], status, w.id, w.startUs);
            }
            w.busy = false;
            any = true;
        }
        return any;
    }

    bool DrainSubmissions() {
        ServeRequest r;
        bool any = false;
        std::lock_guard<std::mutex> g(regMu);
        while (submitQ.Pop(r)) {
            any = true;
            auto it = slotOf.find(r.scene);
            if (it == slotOf.end() || !slots[it->second].live) {
                Complete(r, BEPUGPU_NOT_FOUND, 0, r.submitUs);
                continue;
            }
            Slot& sl = slots[it->second];
            if (sl.s->DeviceBytes() > cfg.device_budget_bytes) {
                Complete(r, BEPUGPU_ADMISSION_REFUSED, 0, r.submitUs);
                continue;
            }
            sl.pending.push_back(r);
            if (!sl.queued && !sl.inFlight) {
                sl.queued = true;
                ready.push_back(it->second);
            }
        }
        return any;
    }

    bool Launch(Wave& w) {
        NvtxRange range("bepugpu_serve_wave");
        std::lock_guard<std::mutex> g(regMu);
        if (ready.empty()) return false;
        w.slotIds.clear();
        w.reqs.clear();
        std::vector<int4> shared, global;
        int sBc = 1, sLc = 1, sMem = 0, gBc = 1, gMem = 0, passes = 0;
        std::vector<int> plain;
        std::deque<int> keep;
        bool noRoom = false;
        while (!ready.empty() && w.slotIds.size() < cfg.max_wave_scenes) {
            int id = ready.front();
            ready.pop_front();
            Slot& sl = slots[id];
            if (!sl.live || sl.pending.empty()) {
                sl.queued = false;
                continue;
            }
            Scene* s = sl.s;
            if (!s->arena) {
                // Once no room could be made, later spilled scenes of this wave
                // wait too (a room search scans every scene).
                if (noRoom || !MakeRoom(s->DeviceBytes())) {
                    noRoom = true;
                    statRoomWaits++;
                    keep.push_back(id);  // waits for room; stays ready
                    continue;
                }
                if (s->Restore(&sink) != BEPUGPU_OK) {
                    SetError(sink.lastError);
                    statRestoreFailures++;
                    keep.push_back(id);
                    continue;
                }
                residentBytes += s->DeviceBytes();
                spilledBytes -= s->DeviceBytes();
                peakResident = std::max(peakResident, residentBytes);
                statRestores++;
                viewsHost[id] = MakeView(*s);
                dirtyViews.push_back(id);
            }
            ServeRequest r = sl.pending.front();
            sl.pending.pop_front();
            sl.queued = false;
            sl.inFlight = true;
            w.slotIds.push_back(id);
            w.reqs.push_back(r);
            if (cfg.batching && s->BatchReady()) {
                const GroupPlan& gp = s->groupPlan;
                passes = std::max(passes, (int)r.steps);
                for (int k = gp.shared.begin; k < gp.shared.end; k++) shared.push_back(make_int4(id, k, (int)r.steps, 0));
                for (int k = gp.global.begin; k < gp.global.end; k++) global.push_back(make_int4(id, k, (int)r.steps, 0));
                if (gp.shared.end > gp.shared.begin) {
                    sBc = std::max(sBc, gp.shared.maxLocal);
                    sLc = std::max(sLc, gp.shared.maxManifolds);
                    sMem = std::max(sMem, gp.shared.maxColourMembers);
                }
                if (gp.global.end > gp.global.begin) {
                    gBc = std::max(gBc, gp.global.maxLocal);
                    gMem = std::max(gMem, gp.global.maxColourMembers);
                }
            } else {
                plain.push_back((int)w.slotIds.size() - 1);
            }
        }
        for (auto it = keep.rbegin(); it != keep.rend(); ++it) ready.push_front(*it);
        if (w.slotIds.empty()) return false;
        // one launch's shared-lane groups must fit a CTA's shared memory together
        if (GroupSmemBytes(true, sBc, sLc) > kGroupSmemBudget + 16 * 1024) {
            for (auto& it : shared) global.push_back(it);
            gBc = std::max(gBc, sBc);
            gMem = std::max(gMem, sMem);
            shared.clear();
        }
        EnsureViewCapacity();
        cudaError_t e = viewsDev ? cudaSuccess : cudaErrorMemoryAllocation;
        // Synchronous copies: any later wave, on any stream, may read these entries.
        if (dirtyViews.size() > 32) {
            if (e == cudaSuccess)
                e = cudaMemcpy(viewsDev, viewsHost.data(), sizeof(SceneView) * viewsHost.size(), cudaMemcpyHostToDevice);
        } else {
            for (int id : dirtyViews)
                if (e == cudaSuccess)
                    e = cudaMemcpy(viewsDev + id, &viewsHost[id], sizeof(SceneView), cudaMemcpyHostToDevice);
        }
        dirtyViews.clear();
        size_t nWork = shared.size() + global.size();
        if (e == cudaSuccess && nWork > w.workCap) {
            if (w.workDev) cudaFree(w.workDev);
            if (w.workHost) cudaFreeHost(w.workHost);
            w.workDev = nullptr;
            w.workHost = nullptr;
            size_t want = std::max(nWork, w.workCap * 2);
            if ((e = cudaMalloc(&w.workDev, sizeof(int4) * want)) == cudaSuccess &&
                (e = cudaMallocHost(&w.workHost, sizeof(int4) * want)) == cudaSuccess)
                w.workCap = want;
            else
                w.workCap = 0;
        }
        w.startUs = NowUs();
        w.id = ++waveCounter;
        if (e == cudaSuccess && nWork) {
            std::copy(shared.begin(), shared.end(), w.workHost);
            std::copy(global.begin(), global.end(), w.workHost + shared.size());
            e = cudaMemcpyAsync(w.workDev, w.workHost, sizeof(int4) * nWork, cudaMemcpyHostToDevice, w.stream);
            if (e == cudaSuccess && !shared.empty()) {
                e = LaunchBatchedGroups(true, viewsDev, w.workDev, (int)shared.size(), p, cfg.flags, sBc, sLc, sMem, 0,
                                        passes, w.stream);
                statLaunches += passes;
            }
            if (e == cudaSuccess && !global.empty()) {
                e = LaunchBatchedGroups(false, viewsDev, w.workDev + shared.size(), (int)global.size(), p, cfg.flags,
                                        gBc, 1, gMem, 0, passes, w.stream);
                statLaunches += passes;
            }
        }
        // one-scene path: each scene's own stream, joined into the wave's event
        for (int k : plain) {
            if (e != cudaSuccess) break;
            Scene* s = slots[w.slotIds[k]].s;
            for (uint32_t st = 0; st < w.reqs[k].steps; st++) {
                if (s->Step(&sink, cfg.dt, cfg.flags) != BEPUGPU_OK) {
                    SetError(sink.lastError);
                    e = cudaErrorUnknown;
                    break;
                }
                statLaunches += s->launchesPerStep;
            }
            if (e == cudaSuccess) e = cudaStreamWaitEvent(w.stream, s->evStop, 0);
        }
        if (e == cudaSuccess) e = cudaEventRecord(w.done, w.stream);
        if (e != cudaSuccess) {
            SetError(std::string("wave launch: ") + cudaGetErrorString(e));
            for (size_t k = 0; k < w.slotIds.size(); k++) {
                slots[w.slotIds[k]].inFlight = false;
                Complete(w.reqs[k], BEPUGPU_CUDA_ERROR, w.id, w.startUs);
            }
            return true;
        }
        w.busy = true;
        statWaves++;
        statWaveScenes += w.slotIds.size();
        return true;
    }

    void Run() {
        cudaSetDevice(ctx->device);
        while (!stop.load(std::memory_order_acquire)) {
            bool progress = FinishWaves();
            progress |= DrainSubmissions();
            for (Wave& w : waves)
                if (!w.busy) {
                    progress |= Launch(w);
                    break;
                }
            if (progress) continue;
            bool busy = false;
            for (Wave& w : waves) busy |= w.busy;
            if (busy) {
                std::this_thread::yield();
            } else {
                std::unique_lock<std::mutex> lk(wakeMu);
                wake.wait_for(lk, std::chrono::microseconds(500));
            }
        }
        for (Wave& w : waves)
            if (w.busy) cudaEventSynchronize(w.done);
    }
};

}  // namespace bepugpu

using namespace bepugpu;

struct bepugpu_server {
    Server* s;
};

extern "C" {

double bepugpu_clock_us(void) { return NowUs(); }

void bepugpu_server_default_config(bepugpu_server_config* out) {
    if (!out) return;
    std::memset(out, 0, sizeof(*out));
    out->device_budget_bytes = 120ull << 30;
    out->max_wave_scenes = 4096;
    out->max_waves_in_flight = 2;
    out->queue_capacity = 1u << 16;
    out->batching = 1;
    out->dt = 1.f / 60.f;
    out->flags = BEPUGPU_STEP_ALL;
}

bepugpu_status bepugpu_server_create(bepugpu_context* c, const bepugpu_server_config* config, bepugpu_server** out) {
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx || !config || !out) return BEPUGPU_INVALID_ARGUMENT;
    if (!Ring<int>::ValidCapacity(config->queue_capacity) || config->max_wave_scenes < 1 ||
        config->max_waves_in_flight < 1 || config->max_waves_in_flight > 4 || !(config->dt > 0) ||
        config->device_budget_bytes == 0) {
        ctx->SetError("server config: queue capacity a power of two >= 2, waves 1..4, dt > 0, a budget");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    cudaSetDevice(ctx->device);
    auto* s = new Server(config->queue_capacity);
    s->ctx = ctx;
    s->sink.device = ctx->device;
    s->sink.smCount = ctx->smCount;
    s->sink.settings = ctx->settings;
    s->cfg = *config;
    s->cfg.flags &= BEPUGPU_STEP_ALL;
    s->p = MakeParams(ctx->settings, config->dt);
    // Let the device's stream-ordered pool keep up to a budget of freed spill
    // memory, so restores reuse it instead of returning it to the driver.
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
        uint64_t keep = config->device_budget_bytes;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    s->waves.resize(config->max_waves_in_flight);
    for (auto& w : s->waves) {
        if (cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming) != cudaSuccess) {
            ctx->SetError("server: stream or event creation failed");
            for (auto& x : s->waves) {
                if (x.stream) cudaStreamDestroy(x.stream);
                if (x.done) cudaEventDestroy(x.done);
            }
            delete s;
            return BEPUGPU_CUDA_ERROR;
        }
    }
    s->worker = std::thread([s] { s->Run(); });
    *out = new bepugpu_server{s};
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_server_destroy(bepugpu_server* h) {
    if (!h) return BEPUGPU_INVALID_ARGUMENT;
    Server* s = h->s;
    s->stop.store(true);
    s->wake.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    bepugpu_status st = BEPUGPU_OK;
    for (auto& sl : s->slots) {
        if (!sl.live) continue;
        if (!sl.s->arena && sl.s->Restore(s->ctx) != BEPUGPU_OK) st = BEPUGPU_OUT_OF_MEMORY;
        sl.s->DropBorrowedSpillBuffer();
        sl.s->server = nullptr;
    }

    for (auto& w : s->waves) {
        if (w.workDev) cudaFree(w.workDev);
        if (w.workHost) cudaFreeHost(w.workHost);
        cudaEventDestroy(w.done);
        cudaStreamDestroy(w.stream);
    }
    if (s->viewsDev) cudaFree(s->viewsDev);
    delete s;
    delete h;
    return st;
}

bepugpu_status bepugpu_server_add_scene(bepugpu_server* h, int32_t scene) {
    if (!h) return BEPUGPU_INVALID_ARGUMENT;
    Server* s = h->s;
    Context* ctx = s->ctx;
    cudaSetDevice(ctx->device);
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) {
        s->SetError("scene " + std::to_string(scene) + " does not exist");
        return BEPUGPU_NOT_FOUND;
    }
    Scene* sc = it->second.get();
    if (sc->server) {
        s->SetError("scene " + std::to_string(scene) + " is already served");
        return BEPUGPU_INVALID_OPERATION;
    }
    if (sc->mode != BEPUGPU_MODE_GRAPH) {
        // a cooperative launch beside other waves' kernels could not count on co-residency
        s->SetError("scene " + std::to_string(scene) + " is in persistent mode; serving takes graph-mode scenes");
        return BEPUGPU_INVALID_OPERATION;
    }
    if (sc->maxBodyReferenced >= sc->b.count || sc->planStale) {
        s->SetError("scene " + std::to_string(scene) + " references bodies it does not hold");
        return BEPUGPU_INVALID_OPERATION;
    }
    if (sc->DeviceBytes() > s->cfg.device_budget_bytes) {
        s->SetError("scene " + std::to_string(scene) + " is larger than the device budget");
        return BEPUGPU_ADMISSION_REFUSED;
    }
    if (sc->asyncPending) {
        cudaStreamSynchronize(sc->stream);
        sc->asyncPending = false;
    }
    if (sc->RefreshDamping(&s->sink, s->cfg.dt) != BEPUGPU_OK ||
        cudaStreamSynchronize(sc->stream) != cudaSuccess) {
        s->SetError(s->sink.lastError);
        return BEPUGPU_CUDA_ERROR;
    }
    std::lock_guard<std::mutex> g(s->regMu);
    int id = (int)s->slots.size();
    Server::Slot sl;
    sl.s = sc;
    sl.lastUse = ++s->useClock;
    s->slots.push_back(sl);
    s->slotOf[scene] = id;
    s->viewsHost.push_back(MakeView(*sc));
    s->dirtyViews.push_back(id);
    sc->server = s;
    s->residentBytes += sc->DeviceBytes();
    // over budget: spill idle scenes, the new one included (it is the most recent)
    if (s->residentBytes > s->cfg.device_budget_bytes) {
        if (!s->MakeRoom(0)) {
            s->SetError("server: no idle scene to spill");
            return BEPUGPU_ADMISSION_REFUSED;
        }
    }
    s->peakResident = std::max(s->peakResident, s->residentBytes);
    return BEPUGPU_OK;
}

// The scene's stream drained, so no spill copy still reads its buffer.
#define CK_SYNC(sc) cudaStreamSynchronize((sc)->stream)

bepugpu_status bepugpu_server_release_scene(bepugpu_server* h, int32_t scene, uint32_t timeout_ms) {
    if (!h) return BEPUGPU_INVALID_ARGUMENT;
    Server* s = h->s;
    cudaSetDevice(s->ctx->device);
    double until = NowUs() + 1000.0 * timeout_ms;
    for (;;) {
        {
            std::lock_guard<std::mutex> g(s->regMu);
            auto it = s->slotOf.find(scene);
            if (it == s->slotOf.end()) return BEPUGPU_NOT_FOUND;
            Server::Slot& sl = s->slots[it->second];
            if (!sl.inFlight && sl.pending.empty()) {
                Scene* sc = sl.s;
                if (!sc->arena) {
                    if (sc->Restore(&s->sink) != BEPUGPU_OK) {
                        s->SetError(s->sink.lastError);
                        return BEPUGPU_OUT_OF_MEMORY;
                    }
                    s->spilledBytes -= sc->DeviceBytes();
                } else {
                    s->residentBytes -= sc->DeviceBytes();
                }
                sl.live = false;
                sl.queued = false;
                s->slotOf.erase(it);
                CK_SYNC(sc);
                sc->DropBorrowedSpillBuffer();
                sc->server = nullptr;
                return BEPUGPU_OK;
            }
        }
        if (NowUs() > until) return BEPUGPU_TIMEOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(200));
    }
}

bepugpu_status bepugpu_serve_submit(bepugpu_server* h, int32_t scene, uint32_t steps, uint64_t tag) {
    if (!h || steps == 0 || steps > 65535) return BEPUGPU_INVALID_ARGUMENT;
    Server* s = h->s;
    ServeRequest r{scene, steps, tag, NowUs()};
    if (!s->submitQ.Push(r)) return BEPUGPU_QUEUE_FULL;
    s->submitted.fetch_add(1, std::memory_order_release);
    s->wake.notify_one();
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_serve_poll(bepugpu_server* h, bepugpu_completion* out, uint32_t max, uint32_t* count) {
    if (!h || (max && !out) || !count) return BEPUGPU_INVALID_ARGUMENT;
    uint32_t n = 0;
    while (n < max && h->s->doneQ.Pop(out[n])) n++;
    *count = n;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_server_drain(bepugpu_server* h, uint32_t timeout_ms) {
    if (!h) return BEPUGPU_INVALID_ARGUMENT;
    Server* s = h->s;
    double until = NowUs() + 1000.0 * timeout_ms;
    while (s->completed.load(std::memory_order_acquire) < s->submitted.load(std::memory_order_acquire)) {
        if (NowUs() > until) return BEPUGPU_TIMEOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_server_stats_get(bepugpu_server* h, bepugpu_server_stats* out) {
    if (!h || !out) return BEPUGPU_INVALID_ARGUMENT;
    Server* s = h->s;
    std::lock_guard<std::mutex> g(s->regMu);
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted.load();
    out->completed = s->completed.load();
    out->waves = s->statWaves;
    out->wave_scenes = s->statWaveScenes;
    out->launches = s->statLaunches;
    out->spills = s->statSpills;
    out->restores = s->statRestores;
    out->room_waits = s->statRoomWaits;
    out->restore_failures = s->statRestoreFailures;
    out->resident_bytes = s->residentBytes;
    out->peak_resident_bytes = s->peakResident;
    out->spilled_bytes = s->spilledBytes;
    for (auto& sl : s->slots)
        if (sl.live) {
            out->scenes++;
            if (sl.s->arena) out->resident_scenes++;
        }
    return BEPUGPU_OK;
}

const char* bepugpu_server_last_error(bepugpu_server* h) {
    if (!h) return "";
    static thread_local std::string copy;
    std::lock_guard<std::mutex> g(h->s->errMu);
    copy = h->s->lastError;
    return copy.c_str();
}

}  // extern "C"
