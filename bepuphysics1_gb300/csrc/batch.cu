// Batched stepping: many scenes advanced in one launch.
//
// The reference's analogue is ParallelSpaceTestDemo.cs:24-64: independent
// Spaces updated side by side, each single-threaded.  Here every island group
// of every listed scene is one CTA of one launch (two when some groups keep
// their solve lanes in global memory); a CTA runs its group's `steps` steps
// back to back with the group's bodies and lanes on chip, so one launch
// advances the whole batch by several steps.  The launches are captured in a
// CUDA graph and reused while the scene list, step counts, dt and settings
// stay the same.
//
// A scene joins the batched launch when its whole step is island groups: no
// constraints on the colour-sweep path, no joints, no dynamic body outside a
// group, and no kinematic body whose candidacy or position stage would change
// it (a moving or always-active one, or one settling in the first steps after
// an upload).  Other listed scenes are stepped with their own one-scene path,
// after the batched launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "groups_device.cuh"
#include "solver_device.cuh"

namespace bepugpu {

// One step of one island group of one scene per CTA.  A call of k steps is k
// launches (pass 0..k-1); a work item whose scene asked for fewer steps than
// the launch's pass returns at once.  Steps run as separate launches rather
// than a loop inside the CTA: the loop keeps the step's body state live across
// iterations and pushes the kernel past the register file into spills.
template <bool kShared>
__device__ __forceinline__ void BatchGroupStep(const SceneView* __restrict__ views, const int4* __restrict__ work,
                                               const StepParams& p, uint32_t flags, int Bc, int Lc, int pass,
                                               bool nonConvex) {
    extern __shared__ float4 smem[];
    __shared__ SceneView sv;
    const int4 w = work[blockIdx.x];  // scene view, group, steps
    if (pass >= w.z) return;
    {
        const int* src = (const int*)(views + w.x);
        int* dst = (int*)&sv;
        for (int i = threadIdx.x; i < (int)(sizeof(SceneView) / sizeof(int)); i += blockDim.x) dst[i] = src[i];
    }
    __syncthreads();
    const GroupDesc g = sv.t.groups[w.y];
    GroupStep<false, kShared, false>(sv.m, sv.b, JointSoA{}, p, flags, sv.t, g, Bc, Lc, 0, smem, nullptr, nonConvex);
}
template <bool kShared>
__global__ void k_batch_groups(const SceneView* __restrict__ views, const int4* __restrict__ work, StepParams p,
                               uint32_t flags, int Bc, int Lc, int pass, bool nonConvex) {
    BatchGroupStep<kShared>(views, work, p, flags, Bc, Lc, pass, nonConvex);
}
// The same kernel held to 168 registers a thread, for 128-thread CTAs: three
// of them fit an SM's 65,536 registers where the unbounded build's 176 fit
// two; ptxas spills a few bytes outside the sweeps.
template <bool kShared>
__global__ void __maxnreg__(168) k_batch_groups_r168(const SceneView* __restrict__ views,
                                                     const int4* __restrict__ work, StepParams p, uint32_t flags,
                                                     int Bc, int Lc, int pass, bool nonConvex) {
    BatchGroupStep<kShared>(views, work, p, flags, Bc, Lc, pass, nonConvex);
}

namespace {

struct ClassLaunch {
    std::vector<int4> work;
    int Bc = 1, Lc = 1, members = 0;
    bool nonConvex = false;  // shared lanes with room for NONCONVEX manifolds' contact friction
    int4* dev = nullptr;
    size_t cap = 0;
};

struct Batch : BatchEngine {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    SceneView* viewsDev = nullptr;
    size_t viewsCap = 0;
    ClassLaunch shared, global;
    std::vector<int4> islandWork;  // the island stage of scenes with islands (AddIslandWork)
    int4* islandDev = nullptr;
    size_t islandCap = 0;
    cudaGraphExec_t graph = nullptr;
    // key of the cached graph
    std::vector<int32_t> keyScenes;
    std::vector<uint32_t> keySteps;
    std::vector<uint64_t> keyVersions;
    std::vector<uint8_t> keyReady;
    float keyDt = 0.f;
    uint32_t keyFlags = 0;
    int keyThreads = 0;
    bepugpu_settings keySettings{};
    uint32_t launches = 0;

    ~Batch() override {
        if (graph) cudaGraphExecDestroy(graph);
        if (viewsDev) cudaFree(viewsDev);
        if (shared.dev) cudaFree(shared.dev);
        if (global.dev) cudaFree(global.dev);
        if (islandDev) cudaFree(islandDev);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
        if (stream) cudaStreamDestroy(stream);
    }
};

int ThreadsFor(int members, int override_) {
    if (override_ > 0) return override_;
    int t = ((members + 31) / 32) * 32;
    return std::min(std::max(t, 32), 256);
}

template <class T>
cudaError_t Ensure(T*& p, size_t& cap, size_t n) {
    if (n <= cap) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    size_t want = std::max(n, cap * 2);
    cudaError_t e = cudaMalloc(&p, sizeof(T) * want);
    cap = e == cudaSuccess ? want : 0;
    return e;
}

template <bool kShared>
cudaError_t LaunchBatchClass(Batch& bt, ClassLaunch& c, const StepParams& p, uint32_t flags, int threads,
                             int passes, int firstPass = 0) {
    if (c.work.empty()) return cudaSuccess;
    bt.launches += passes;
    return LaunchBatchedGroups(kShared, bt.viewsDev, c.dev, (int)c.work.size(), p, flags, c.Bc, c.Lc, c.members,
                               threads, passes, bt.stream, c.nonConvex, firstPass);
}

}  // namespace

cudaError_t LaunchBatchedGroups(bool shared, const SceneView* views, const int4* work, int n, const StepParams& p,
                                uint32_t flags, int Bc, int Lc, int members, int threads, int passes,
                                cudaStream_t stream, bool nonConvex, int firstPass) {
    if (n <= 0) return cudaSuccess;
    size_t smemBytes = GroupSmemBytes(shared, Bc, Lc, 0, nonConvex);
    const int T = ThreadsFor(members, threads);
    auto kernel = T == 128 ? (shared ? k_batch_groups_r168<true> : k_batch_groups_r168<false>)
                           : (shared ? k_batch_groups<true> : k_batch_groups<false>);
    if (smemBytes > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smemBytes);
        if (e != cudaSuccess) return e;
    }
    for (int pass = firstPass; pass < firstPass + passes; pass++) {
        kernel<<<(unsigned)n, T, smemBytes, stream>>>(views, work, p, flags, Bc, Lc, pass, nonConvex);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

SceneView MakeView(const Scene& s) {
    SceneView v;
    v.m = s.m;
    v.b = s.b;
    v.t.groups = s.groupDescDev;
    v.t.bodies = s.groupBodiesDev;
    v.t.refs = s.groupRefsDev;
    v.t.colourOffsets = s.groupColourOffsetsDev;
    v.t.jointRefs = nullptr;  // batched scenes hold no joints
    v.t.jointColourOffsets = nullptr;
    FillIslandView(s, v.isl);
    return v;
}

bool Scene::BatchReady(uint32_t flags) const {
    // scenes with islands batch while no kinematic body can wake an island
    return SweepEmpty() && jointCount == 0 && generatedCount == 0 && !kin.Needed(StageFlags(flags)) &&
           (!islands || !IslandWakesPossible(this));
}

}  // namespace bepugpu

using namespace bepugpu;

static bepugpu_status BatchStep(bepugpu_context* c, const int32_t* scenes, const uint32_t* stepsEach, uint32_t steps,
                                uint32_t count, float dt, uint32_t flags) {
    NvtxRange range("bepugpu_batch_step");
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if ((count && !scenes) || !(dt > 0)) {
        ctx->SetError("batch: scenes must be given and dt must be positive");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    flags &= BEPUGPU_STEP_ALL;
    if (!ctx->batch) {
        auto* b = new Batch();
        if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess) {
            delete b;
            ctx->SetError("batch: stream or event creation failed");
            return BEPUGPU_CUDA_ERROR;
        }
        ctx->batch.reset(b);
    }
    Batch& bt = *static_cast<Batch*>(ctx->batch.get());
    std::vector<Scene*> list(count);
    std::vector<uint32_t> stepCount(count);
    // A stamp per call marks the listed scenes (duplicate check in one pass);
    // the epoch advances whether or not the call succeeds.
    struct EpochBump {
        Context* c;
        ~EpochBump() { c->batchEpoch++; }
    } bump{ctx};
    std::vector<uint64_t> versions(count);
    std::vector<uint8_t> ready(count);  // joins the batched launch
    for (uint32_t i = 0; i < count; i++) {
        auto it = ctx->scenes.find(scenes[i]);
        if (it == ctx->scenes.end()) {
            ctx->SetError("batch: scene %d does not exist", scenes[i]);
            return BEPUGPU_NOT_FOUND;
        }
        Scene* s = it->second.get();
        if (s->server) {
            ctx->SetError("batch: scene %d is served; release it first", scenes[i]);
            return BEPUGPU_INVALID_OPERATION;
        }
        uint32_t k = stepsEach ? stepsEach[i] : steps;
        if (k > 65535) {
            ctx->SetError("batch: at most 65535 steps per call");
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if (s->maxBodyReferenced >= s->b.count || s->planStale) {
            ctx->SetError("batch: scene %d references body %d of %d or changed dynamic bodies since its constraints "
                          "were uploaded", scenes[i], s->maxBodyReferenced, s->b.count);
            return BEPUGPU_INVALID_OPERATION;
        }
        if (s->batchStamp == ctx->batchEpoch + 1) {
            ctx->SetError("batch: scene %d is listed twice", scenes[i]);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        s->batchStamp = ctx->batchEpoch + 1;
        list[i] = s;
        stepCount[i] = k;
        versions[i] = s->version;
        ready[i] = s->BatchReady(flags) ? 1 : 0;
        if (s->asyncPending) {  // a one-scene step may still run on the scene's stream
            if (cudaStreamSynchronize(s->stream) != cudaSuccess) {
                ctx->SetError("batch: scene %d stream failed", scenes[i]);
                return BEPUGPU_CUDA_ERROR;
            }
            s->asyncPending = false;
        }
        bepugpu_status st = s->RefreshDamping(ctx, dt);
        if (st != BEPUGPU_OK) return st;
    }
    StepParams p = MakeParams(ctx->settings, dt);
    bool same = bt.graph && bt.keyDt == dt && bt.keyFlags == flags && bt.keyThreads == ctx->batchThreads &&
                std::memcmp(&bt.keySettings, &ctx->settings, sizeof(bepugpu_settings)) == 0 &&
                bt.keyScenes.size() == count && std::equal(scenes, scenes + count, bt.keyScenes.begin()) &&
                bt.keySteps == stepCount && bt.keyVersions == versions && bt.keyReady == ready;
    cudaError_t e = cudaSuccess;
    if (!same) {
        if (bt.graph) {
            cudaGraphExecDestroy(bt.graph);
            bt.graph = nullptr;
        }
        std::vector<SceneView> views;
        int passes = 0;  // launches per class: the most steps any batched scene asked for
        bt.shared = ClassLaunch{{}, 1, 1, 0, false, bt.shared.dev, bt.shared.cap};
        bt.global = ClassLaunch{{}, 1, 1, 0, false, bt.global.dev, bt.global.cap};
        bt.islandWork.clear();
        for (uint32_t i = 0; i < count; i++) {
            Scene* s = list[i];
            if (!ready[i] || stepCount[i] == 0) continue;
            passes = std::max(passes, (int)stepCount[i]);
            const GroupPlan& g = s->groupPlan;
            const int vi = (int)views.size();
            views.push_back(MakeView(*s));
            if (flags & BEPUGPU_STEP_DEACTIVATION) AddIslandWork(*s, vi, (int)stepCount[i], bt.islandWork);
            for (int k = g.shared.begin; k < g.shared.end; k++)
                bt.shared.work.push_back(make_int4(vi, k, (int)stepCount[i], 0));
            for (int k = g.global.begin; k < g.global.end; k++)
                bt.global.work.push_back(make_int4(vi, k, (int)stepCount[i], 0));
            if (g.shared.end > g.shared.begin) {
                bt.shared.Bc = std::max(bt.shared.Bc, g.shared.maxLocal);
                bt.shared.Lc = std::max(bt.shared.Lc, g.shared.maxManifolds);
                bt.shared.members = std::max(bt.shared.members, g.shared.maxColourMembers);
                bt.shared.nonConvex = bt.shared.nonConvex || g.nonConvexLanes;
            }
            if (g.global.end > g.global.begin) {
                bt.global.Bc = std::max(bt.global.Bc, g.global.maxLocal);
                bt.global.members = std::max(bt.global.members, g.global.maxColourMembers);
            }
        }
        // the shared-lane groups of different scenes must fit one launch's budget together
        const size_t sharedBytes = GroupSmemBytes(true, bt.shared.Bc, bt.shared.Lc, 0, bt.shared.nonConvex);
        if (sharedBytes > kGroupSmemBudget + 16 * 1024) {
            ctx->SetError("batch: shared-lane groups need %zu bytes of shared memory", sharedBytes);
            return BEPUGPU_INVALID_OPERATION;
        }
        if ((e = Ensure(bt.viewsDev, bt.viewsCap, std::max<size_t>(views.size(), 1))) ||
            (e = Ensure(bt.shared.dev, bt.shared.cap, std::max<size_t>(bt.shared.work.size(), 1))) ||
            (e = Ensure(bt.global.dev, bt.global.cap, std::max<size_t>(bt.global.work.size(), 1))) ||
            (e = Ensure(bt.islandDev, bt.islandCap, std::max<size_t>(bt.islandWork.size(), 1)))) {
            ctx->SetError("batch tables: %s", cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? BEPUGPU_OUT_OF_MEMORY : BEPUGPU_CUDA_ERROR;
        }
        if ((!views.empty() && (e = cudaMemcpyAsync(bt.viewsDev, views.data(), sizeof(SceneView) * views.size(),
                                                    cudaMemcpyHostToDevice, bt.stream))) ||
            (!bt.shared.work.empty() &&
             (e = cudaMemcpyAsync(bt.shared.dev, bt.shared.work.data(), sizeof(int4) * bt.shared.work.size(),
                                  cudaMemcpyHostToDevice, bt.stream))) ||
            (!bt.global.work.empty() &&
             (e = cudaMemcpyAsync(bt.global.dev, bt.global.work.data(), sizeof(int4) * bt.global.work.size(),
                                  cudaMemcpyHostToDevice, bt.stream))) ||
            (!bt.islandWork.empty() &&
             (e = cudaMemcpyAsync(bt.islandDev, bt.islandWork.data(), sizeof(int4) * bt.islandWork.size(),
                                  cudaMemcpyHostToDevice, bt.stream))) ||
            (e = cudaStreamSynchronize(bt.stream))) {
            ctx->SetError("batch tables: %s", cudaGetErrorString(e));
            return BEPUGPU_CUDA_ERROR;
        }
        bt.launches = 0;
        if ((e = cudaStreamBeginCapture(bt.stream, cudaStreamCaptureModeThreadLocal))) {
            ctx->SetError("batch capture: %s", cudaGetErrorString(e));
            return BEPUGPU_CUDA_ERROR;
        }
        cudaError_t le = cudaSuccess;
        if (bt.islandWork.empty()) {
            le = LaunchBatchClass<true>(bt, bt.shared, p, flags, ctx->batchThreads, passes);
            if (le == cudaSuccess) le = LaunchBatchClass<false>(bt, bt.global, p, flags, ctx->batchThreads, passes);
        } else {
            // step by step: the island stage of step k before any group's step k
            for (int pass = 0; pass < passes && le == cudaSuccess; pass++) {
                le = LaunchBatchedIslands(bt.viewsDev, bt.islandDev, (int)bt.islandWork.size(), p,
                                          ctx->settings.maximum_deactivation_attempts_per_frame, pass, bt.stream);
                bt.launches++;
                if (le == cudaSuccess) le = LaunchBatchClass<true>(bt, bt.shared, p, flags, ctx->batchThreads, 1, pass);
                if (le == cudaSuccess) le = LaunchBatchClass<false>(bt, bt.global, p, flags, ctx->batchThreads, 1, pass);
            }
        }
        cudaGraph_t graph = nullptr;
        e = cudaStreamEndCapture(bt.stream, &graph);
        if (le != cudaSuccess || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            ctx->SetError("batch launch: %s", cudaGetErrorString(le != cudaSuccess ? le : e));
            return BEPUGPU_CUDA_ERROR;
        }
        e = cudaGraphInstantiate(&bt.graph, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) {
            bt.graph = nullptr;
            ctx->SetError("batch graph: %s", cudaGetErrorString(e));
            return BEPUGPU_CUDA_ERROR;
        }
        bt.keyScenes.assign(scenes, scenes + count);
        bt.keySteps = stepCount;
        bt.keyVersions = versions;
        bt.keyReady = ready;
        bt.keyDt = dt;
        bt.keyFlags = flags;
        bt.keyThreads = ctx->batchThreads;
        bt.keySettings = ctx->settings;
    }
    if ((e = cudaEventRecord(bt.ev0, bt.stream)) || (e = cudaGraphLaunch(bt.graph, bt.stream)) ||
        (e = cudaEventRecord(bt.ev1, bt.stream)) || (e = cudaStreamSynchronize(bt.stream))) {
        ctx->SetError("batch step: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    uint32_t launches = bt.launches;
    // Scenes outside the batched launch take their own path, step by step.
    for (uint32_t i = 0; i < count; i++) {
        Scene* s = list[i];
        if (ready[i]) {
            for (uint32_t k = 0; k < stepCount[i]; k++) s->kin.Advance(flags);
            continue;
        }
        for (uint32_t k = 0; k < stepCount[i]; k++) {
            bepugpu_status st = s->Step(ctx, dt, flags);
            if (st != BEPUGPU_OK) return st;
            launches += s->launchesPerStep;
        }
        if (stepCount[i] && cudaStreamSynchronize(s->stream) != cudaSuccess) {
            ctx->SetError("batch: one-scene steps failed");
            return BEPUGPU_CUDA_ERROR;
        }
        s->asyncPending = false;
    }
    ctx->lastLaunches = launches;
    cudaEventElapsedTime(&ctx->lastMs, bt.ev0, bt.ev1);
    return BEPUGPU_OK;
}

extern "C" bepugpu_status bepugpu_batch_step(bepugpu_context* c, const int32_t* scenes, uint32_t count, float dt,
                                             uint32_t steps, uint32_t flags) {
    return BatchStep(c, scenes, nullptr, steps, count, dt, flags);
}

extern "C" bepugpu_status bepugpu_batch_step_each(bepugpu_context* c, const int32_t* scenes, const uint32_t* steps,
                                                  uint32_t count, float dt, uint32_t flags) {
    if (count && !steps) return BEPUGPU_INVALID_ARGUMENT;
    return BatchStep(c, scenes, steps, 0, count, dt, flags);
}

extern "C" bepugpu_status bepugpu_set_batch_threads(bepugpu_context* c, int32_t threads) {
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    if (threads != 0 && (threads < 32 || threads > 256 || threads % 32)) {
        ctx->SetError("batch threads must be 0 or a multiple of 32 in [32, 256]");
        return BEPUGPU_INVALID_ARGUMENT;
    }
    ctx->batchThreads = threads;
    return BEPUGPU_OK;
}
