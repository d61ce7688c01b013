// Serving: step requests for many resident scenes, batched continuously.
//
// Submitters push {scene, steps, tag} into a lock-free ring (ring.h).  One
// worker thread owns everything else: per-scene FIFOs of requests, the ready
// order (scenes whose head request waits, in arrival order), residency under
// the device budget with least-recently-used spills to pinned host memory,
// and up to four waves in flight.  A wave takes every ready scene that is not
// already on the device (one request each) and launches, on the wave's own
// stream, the batched group kernel over all their island groups (batch.cu;
// one launch per step, up to the most steps a request of the wave asked for,
// CTAs of requests with fewer steps returning at once) plus the one-scene
// path for scenes the batched kernel cannot take.  Completion of a
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
#include <map>
#include <mutex>
#include <set>
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

// Pinned host memory for spill buffers, carved from large slabs.  Pinning
// costs about as much per byte as a copy, so it is paid once, when the served
// set first outgrows the device budget, and not on a request's path.
// Returned buffers are reused best fit (within twice the size asked).
class HostPool {
  public:
    ~HostPool() {
        for (void* p : slabs_) cudaFreeHost(p);
    }
    void* Take(size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        auto it = free_.lower_bound(bytes);
        if (it != free_.end() && it->first <= 2 * bytes) {
            void* p = it->second;
            size_[p] = it->first;
            free_.erase(it);
            return p;
        }
        if (left_ < bytes) {
            if (left_ >= (64u << 10)) Give(cur_, left_);
            size_t slab = std::max(bytes, kSlab);
            void* p = nullptr;
            if (cudaMallocHost(&p, slab) != cudaSuccess) return nullptr;
            slabs_.push_back(p);
            pinned_ += slab;
            cur_ = (char*)p;
            left_ = slab;
        }
        void* p = cur_;
        cur_ += bytes;
        left_ -= bytes;
        size_[p] = bytes;
        return p;
    }
    void Give(void* p) {
        auto it = size_.find(p);
        if (it == size_.end()) return;
        free_.emplace(it->second, p);
        size_.erase(it);
    }
    size_t Pinned() const { return pinned_; }
    void Abandon() { slabs_.clear(); }

  private:
    void Give(char* p, size_t bytes) { free_.emplace(bytes, p); }
    static constexpr size_t kSlab = 256u << 20;
    std::vector<void*> slabs_;
    std::multimap<size_t, void*> free_;
    std::unordered_map<void*, size_t> size_;
    char* cur_ = nullptr;
    size_t left_ = 0, pinned_ = 0;
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
    // resident scenes by last use; an entry whose scene has queued or running
    // requests is skipped (and dropped) when victims are picked, and comes back
    // when the scene's wave finishes
    std::set<std::pair<uint64_t, int>> lru;
    HostPool hostPool;
    bool lending = false;  // the served set outgrew the budget: every scene holds a spill buffer
    uint64_t servedBytes = 0;

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
    double usSpill = 0, usRestore = 0;
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

    void Touch(int id) {
        Slot& sl = slots[id];
        lru.erase({sl.lastUse, id});
        sl.lastUse = ++useClock;
        lru.insert({sl.lastUse, id});
    }

    // Every served scene gets a pinned spill buffer from the pool.
    void LendSpillBuffers(Scene* only) {
        for (Slot& sl : slots) {
            if (!sl.live || (only && sl.s != only) || sl.s->spillHost) continue;
            sl.s->LendSpillBuffer(hostPool.Take(sl.s->arenaBytes));
        }
    }

    // Spill least recently used idle scenes until `need` more bytes fit.  The
    // victims' copies run together; their streams are drained before this
    // returns, so the freed device memory is back in the pool for restores.
    bool MakeRoom(size_t need) {
        if (residentBytes + need <= cfg.device_budget_bytes) return true;
        double t0 = NowUs();
        std::vector<Scene*> spilled;
        bool ok = true;
        while (residentBytes + need > cfg.device_budget_bytes) {
            if (lru.empty()) {
                ok = false;
                break;
            }
            const int id = lru.begin()->second;
            lru.erase(lru.begin());
            const Slot& v = slots[id];
            if (!v.live || !v.s->arena || v.inFlight || !v.pending.empty()) continue;
            Scene* s = v.s;
            size_t bytes = s->DeviceBytes();
            if (s->Spill(&sink, false) != BEPUGPU_OK) {
                SetError(sink.lastError);
                ok = false;
                break;
            }
            spilled.push_back(s);
            residentBytes -= bytes;
            spilledBytes += bytes;
            statSpills++;
        }
        for (Scene* s : spilled)
            if (cudaStreamSynchronize(s->stream) != cudaSuccess) {
                SetError("spill copy failed");
                ok = false;
            }
        usSpill += NowUs() - t0;
        return ok;
    }

    cudaError_t EnsureViewCapacity() {
        if (viewsCap >= viewsHost.size()) return cudaSuccess;
        size_t want = std::max<size_t>(viewsHost.size(), viewsCap * 2);
        SceneView* d = nullptr;
        const cudaError_t e = cudaMalloc(&d, sizeof(SceneView) * want);
        if (e != cudaSuccess) return e;
        if (viewsDev) {
            cudaDeviceSynchronize();  // no wave reads the old table any more
            cudaFree(viewsDev);
        }
        viewsDev = d;
        viewsCap = want;
        dirtyViews.clear();
        for (int i = 0; i < (int)viewsHost.size(); i++) dirtyViews.push_back(i);
        return cudaSuccess;
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
                Touch(w.slotIds[k]);
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
        std::vector<int4> shared, global, islandW;  // islandW: the island stage of scenes with islands
        int sBc = 1, sLc = 1, sMem = 0, gBc = 1, gMem = 0, passes = 0;
        bool sNonConvex = false;  // a shared-lane group holds a NONCONVEX manifold
        std::vector<int> plain;
        std::deque<int> keep;
        std::vector<Scene*> restored;  // copies in flight on their scenes' streams
        // The wave's scenes first, then room for all of its spilled ones at
        // once (one round of spill copies), then their restores.
        std::vector<int> chosen;
        size_t need = 0;
        while (!ready.empty() && chosen.size() < cfg.max_wave_scenes) {
            int id = ready.front();
            ready.pop_front();
            Slot& sl = slots[id];
            if (!sl.live || sl.pending.empty()) {
                sl.queued = false;
                continue;
            }
            chosen.push_back(id);
            if (!sl.s->arena) need += sl.s->DeviceBytes();
        }
        if (need) MakeRoom(need);  // may free less; the scenes that do not fit wait
        bool noRoom = false;
        for (size_t c = 0;; c++) {
            int id;
            if (c < chosen.size()) {
                id = chosen[c];
            } else {
                // Some chosen scenes wait for room: resident scenes queued behind
                // them fill the wave (they need none), so the scenes that hold
                // the device keep finishing and become spill victims.
                if (ready.empty() || w.slotIds.size() >= cfg.max_wave_scenes) break;
                id = ready.front();
                ready.pop_front();
                Slot& sl = slots[id];
                if (!sl.live || sl.pending.empty()) {
                    sl.queued = false;
                    continue;
                }
                if (!sl.s->arena) {
                    statRoomWaits++;
                    keep.push_back(id);
                    continue;
                }
            }
            Slot& sl = slots[id];
            Scene* s = sl.s;
            if (!s->arena) {
                // Once one spilled scene finds no room, later ones of this wave
                // wait too, so they keep their order.
                if (noRoom || residentBytes + s->DeviceBytes() > cfg.device_budget_bytes) {
                    noRoom = true;
                    statRoomWaits++;
                    keep.push_back(id);  // waits for room; stays ready
                    continue;
                }
                const double t0 = NowUs();
                const bepugpu_status rs = s->Restore(&sink, nullptr, false);
                usRestore += NowUs() - t0;
                if (rs != BEPUGPU_OK) {
                    SetError(sink.lastError);
                    statRestoreFailures++;
                    keep.push_back(id);
                    continue;
                }
                restored.push_back(s);
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
            if (cfg.batching && s->BatchReady(cfg.flags)) {
                for (uint32_t k = 0; k < r.steps; k++) s->kin.Advance(cfg.flags);
                if (cfg.flags & BEPUGPU_STEP_DEACTIVATION) AddIslandWork(*s, id, (int)r.steps, islandW);
                const GroupPlan& gp = s->groupPlan;
                passes = std::max(passes, (int)r.steps);
                for (int k = gp.shared.begin; k < gp.shared.end; k++) shared.push_back(make_int4(id, k, (int)r.steps, 0));
                for (int k = gp.global.begin; k < gp.global.end; k++) global.push_back(make_int4(id, k, (int)r.steps, 0));
                if (gp.shared.end > gp.shared.begin) {
                    sBc = std::max(sBc, gp.shared.maxLocal);
                    sLc = std::max(sLc, gp.shared.maxManifolds);
                    sMem = std::max(sMem, gp.shared.maxColourMembers);
                    sNonConvex = sNonConvex || gp.nonConvexLanes;
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
        cudaError_t e = cudaSuccess;
        const char* failedAt = "";
        auto check = [&](cudaError_t r, const char* at) {
            if (e == cudaSuccess && r != cudaSuccess) {
                e = r;
                failedAt = at;
            }
        };
        if (!restored.empty()) {
            const double t0 = NowUs();
            for (Scene* s : restored)
                if (e == cudaSuccess) check(cudaStreamSynchronize(s->stream), "restore copy");
            usRestore += NowUs() - t0;
        }
        if (w.slotIds.empty()) return false;
        // one launch's shared-lane groups must fit a CTA's shared memory together
        if (GroupSmemBytes(true, sBc, sLc, 0, sNonConvex) > kGroupSmemBudget + 16 * 1024) {
            for (auto& it : shared) global.push_back(it);
            gBc = std::max(gBc, sBc);
            gMem = std::max(gMem, sMem);
            shared.clear();
        }
        if (e == cudaSuccess) check(EnsureViewCapacity(), "scene table allocation");
        // Synchronous copies: any later wave, on any stream, may read these entries.
        if (dirtyViews.size() > 32) {
            if (e == cudaSuccess)
                check(cudaMemcpy(viewsDev, viewsHost.data(), sizeof(SceneView) * viewsHost.size(),
                                 cudaMemcpyHostToDevice), "scene table copy");
        } else {
            for (int id : dirtyViews)
                if (e == cudaSuccess)
                    check(cudaMemcpy(viewsDev + id, &viewsHost[id], sizeof(SceneView), cudaMemcpyHostToDevice),
                          "scene table copy");
        }
        dirtyViews.clear();
        size_t nWork = shared.size() + global.size() + islandW.size();
        if (e == cudaSuccess && nWork > w.workCap) {
            if (w.workDev) cudaFree(w.workDev);
            if (w.workHost) cudaFreeHost(w.workHost);
            w.workDev = nullptr;
            w.workHost = nullptr;
            size_t want = std::max(nWork, w.workCap * 2);
            check(cudaMalloc(&w.workDev, sizeof(int4) * want), "work list allocation");
            if (e == cudaSuccess) check(cudaMallocHost(&w.workHost, sizeof(int4) * want), "work list allocation");
            if (e == cudaSuccess)
                w.workCap = want;
            else
                w.workCap = 0;
        }
        w.startUs = NowUs();
        w.id = ++waveCounter;
        if (e == cudaSuccess && nWork) {
            std::copy(shared.begin(), shared.end(), w.workHost);
            std::copy(global.begin(), global.end(), w.workHost + shared.size());
            std::copy(islandW.begin(), islandW.end(), w.workHost + shared.size() + global.size());
            check(cudaMemcpyAsync(w.workDev, w.workHost, sizeof(int4) * nWork, cudaMemcpyHostToDevice, w.stream),
                  "work list copy");
            // with islands, step by step: the island stage of step k before any group's step k
            const int rounds = islandW.empty() ? 1 : passes, per = islandW.empty() ? passes : 1;
            for (int round = 0; round < rounds && e == cudaSuccess; round++) {
                if (!islandW.empty()) {
                    const int attempts = sink.settings.maximum_deactivation_attempts_per_frame;
                    check(LaunchBatchedIslands(viewsDev, w.workDev + shared.size() + global.size(),
                                               (int)islandW.size(), p, attempts, round, w.stream),
                          "island launch");
                    statLaunches++;
                }
                if (e == cudaSuccess && !shared.empty()) {
                    check(LaunchBatchedGroups(true, viewsDev, w.workDev, (int)shared.size(), p, cfg.flags, sBc, sLc,
                                              sMem, (int)cfg.threads, per, w.stream, sNonConvex, round),
                          "group launch");
                    statLaunches += per;
                }
                if (e == cudaSuccess && !global.empty()) {
                    check(LaunchBatchedGroups(false, viewsDev, w.workDev + shared.size(), (int)global.size(), p,
                                              cfg.flags, gBc, 1, gMem, (int)cfg.threads, per, w.stream, false,
                                              round),
                          "group launch");
                    statLaunches += per;
                }
            }
        }
        // one-scene path: each scene's own stream, joined into the wave's event
        bool stepFailed = false;
        for (int k : plain) {
            if (e != cudaSuccess) break;
            Scene* s = slots[w.slotIds[k]].s;
            for (uint32_t st = 0; st < w.reqs[k].steps; st++) {
                if (s->Step(&sink, cfg.dt, cfg.flags) != BEPUGPU_OK) {
                    SetError("wave step: " + sink.lastError);
                    stepFailed = true;
                    check(cudaErrorUnknown, "step");
                    break;
                }
                statLaunches += s->launchesPerStep;
            }
            if (e == cudaSuccess) check(cudaStreamWaitEvent(w.stream, s->evStop, 0), "wave join");
        }
        if (e == cudaSuccess) check(cudaEventRecord(w.done, w.stream), "wave event");
        if (e != cudaSuccess) {
            if (!stepFailed) SetError(std::string("wave launch (") + failedAt + "): " + cudaGetErrorString(e));
            for (size_t k = 0; k < w.slotIds.size(); k++) {
                Slot& sl = slots[w.slotIds[k]];
                sl.inFlight = false;
                Touch(w.slotIds[k]);
                if (!sl.pending.empty() && !sl.queued) {
                    sl.queued = true;
                    ready.push_back(w.slotIds[k]);
                }
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

// Stops the worker (waves on the device finish first), restores spilled
// scenes and hands every scene back to its context.
bepugpu_status Shutdown(Server* s) {
    s->stop.store(true);
    s->wake.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->ctx->device);
    bepugpu_status st = BEPUGPU_OK;
    bool stranded = false;
    for (auto& sl : s->slots) {
        if (!sl.live) continue;
        if (!sl.s->arena && sl.s->Restore(s->ctx) != BEPUGPU_OK) {
            st = BEPUGPU_OUT_OF_MEMORY;
            // still spilled: its data must outlive the server's pool
            if (!sl.s->OwnSpillBuffer()) stranded = true;
        }
        sl.s->DropBorrowedSpillBuffer();
        sl.s->server = nullptr;
    }
    if (stranded) s->hostPool.Abandon();  // a scene still reads a slab: keep them all

    for (auto& w : s->waves) {
        if (w.workDev) cudaFree(w.workDev);
        if (w.workHost) cudaFreeHost(w.workHost);
        cudaEventDestroy(w.done);
        cudaStreamDestroy(w.stream);
    }
    if (s->viewsDev) cudaFree(s->viewsDev);
    s->ctx->heap->Hold(false);
    delete s;
    return st;
}

}  // namespace bepugpu

using namespace bepugpu;

struct bepugpu_server {
    Server* s;  // null once the server's context was destroyed
};

namespace bepugpu {
void ShutdownServers(Context* ctx) {
    for (bepugpu_server* h : ctx->servers) {
        Shutdown(h->s);
        h->s = nullptr;
    }
    ctx->servers.clear();
}
}  // namespace bepugpu

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
        config->device_budget_bytes == 0 ||
        (config->threads != 0 && (config->threads < 32 || config->threads > 256 || config->threads % 32))) {
        ctx->SetError("server config: queue capacity a power of two >= 2, waves 1..4, dt > 0, a budget, "
                      "threads 0 or a multiple of 32 in [32, 256]");
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
    ctx->heap->Hold(true);
    s->waves.resize(config->max_waves_in_flight);
    for (auto& w : s->waves) {
        if (cudaStreamCreateWithFlags(&w.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming) != cudaSuccess) {
            ctx->SetError("server: stream or event creation failed");
            for (auto& x : s->waves) {
                if (x.stream) cudaStreamDestroy(x.stream);
                if (x.done) cudaEventDestroy(x.done);
            }
            ctx->heap->Hold(false);
            delete s;
            return BEPUGPU_CUDA_ERROR;
        }
    }
    s->worker = std::thread([s] { s->Run(); });
    *out = new bepugpu_server{s};
    ctx->servers.push_back(*out);
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_server_destroy(bepugpu_server* h) {
    if (!h) return BEPUGPU_INVALID_ARGUMENT;
    bepugpu_status st = BEPUGPU_OK;
    if (h->s) {
        auto& list = h->s->ctx->servers;
        list.erase(std::remove(list.begin(), list.end(), h), list.end());
        st = Shutdown(h->s);
    }
    delete h;
    return st;
}

#define SERVER_CHECK(h)                                               \
    do {                                                              \
        if (!(h)) return BEPUGPU_INVALID_ARGUMENT;                    \
        if (!(h)->s) return BEPUGPU_INVALID_OPERATION; /* context gone */ \
    } while (0)



bepugpu_status bepugpu_server_add_scene(bepugpu_server* h, int32_t scene) {
    SERVER_CHECK(h);
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
    s->lru.insert({sl.lastUse, id});
    s->servedBytes += sc->DeviceBytes();
    // Once the served scenes outgrow the budget any of them may be spilled:
    // all get pinned spill buffers now rather than on a request's path.
    if (s->servedBytes > s->cfg.device_budget_bytes) {
        s->LendSpillBuffers(s->lending ? sc : nullptr);
        s->lending = true;
    }
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
    SERVER_CHECK(h);
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
                s->lru.erase({sl.lastUse, it->second});
                s->servedBytes -= sc->DeviceBytes();
                s->slotOf.erase(it);
                CK_SYNC(sc);
                if (sc->spillHostBorrowed) s->hostPool.Give(sc->spillHost);
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
    SERVER_CHECK(h);
    if (steps == 0 || steps > 65535) return BEPUGPU_INVALID_ARGUMENT;
    Server* s = h->s;
    ServeRequest r{scene, steps, tag, NowUs()};
    if (!s->submitQ.Push(r)) return BEPUGPU_QUEUE_FULL;
    s->submitted.fetch_add(1, std::memory_order_release);
    s->wake.notify_one();
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_serve_poll(bepugpu_server* h, bepugpu_completion* out, uint32_t max, uint32_t* count) {
    SERVER_CHECK(h);
    if ((max && !out) || !count) return BEPUGPU_INVALID_ARGUMENT;
    uint32_t n = 0;
    while (n < max && h->s->doneQ.Pop(out[n])) n++;
    *count = n;
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_server_drain(bepugpu_server* h, uint32_t timeout_ms) {
    SERVER_CHECK(h);
    Server* s = h->s;
    double until = NowUs() + 1000.0 * timeout_ms;
    while (s->completed.load(std::memory_order_acquire) < s->submitted.load(std::memory_order_acquire)) {
        if (NowUs() > until) return BEPUGPU_TIMEOUT;
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
    return BEPUGPU_OK;
}

bepugpu_status bepugpu_server_stats_get(bepugpu_server* h, bepugpu_server_stats* out) {
    SERVER_CHECK(h);
    if (!out) return BEPUGPU_INVALID_ARGUMENT;
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
    out->spill_us = (uint64_t)s->usSpill;
    out->restore_us = (uint64_t)s->usRestore;
    out->pinned_bytes = s->hostPool.Pinned();
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
    if (!h->s) return "the server's context was destroyed";
    static thread_local std::string copy;
    std::lock_guard<std::mutex> g(h->s->errMu);
    copy = h->s->lastError;
    return copy.c_str();
}

}  // extern "C"
