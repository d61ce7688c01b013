// Host-side objects behind the C ABI: contexts and scenes.
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/bepugpu.h"
#include "colouring.h"
#include "joints_device.cuh"
#include "solver_device.cuh"

namespace bepugpu {

struct Context;
struct BatchEngine;
struct Scene;
struct BroadPhaseBuffers;
void ReleaseBroadPhase(Scene* s);  // broadphase.cu
struct Context;
// broadphase.cu: the pair set into device memory (sorted 64-bit keys, lower
// body << 32 | higher), the ascending bitonic sort of 64-bit keys it uses
// (`padded` a power of two from PaddedSize), and a filler of largest keys.
bepugpu_status RunBroadPhase(Context* ctx, Scene* s, float dt, unsigned& found);
const unsigned long long* BroadPhasePairs(const Scene* s);
size_t PaddedSize(size_t n);
void SortKeys(unsigned long long* keys, size_t padded, cudaStream_t st);
void FillKeys(unsigned long long* keys, size_t n, cudaStream_t st);
struct PairBuffers;                // pairs.cu
void ReleasePairs(Scene* s);
struct IslandBuffers;               // islands.cu
struct StepParams;
void ReleaseIslands(Scene* s);
void ApplyIslandViews(Scene* s);    // the body view's island pointers after a rebase
cudaError_t LaunchIslandStage(Scene* s, const StepParams& p, int maxAttempts, cudaStream_t q);
bool IslandWakesPossible(const Scene* s);

// Device memory of a context's scene arenas and staging buffers, carved from
// large cudaMalloc slabs (heap.cu).  Thread-safe: a server's worker spills and
// restores while the caller's thread creates and destroys scenes.
class DeviceHeap {
  public:
    DeviceHeap() = default;
    DeviceHeap(const DeviceHeap&) = delete;
    DeviceHeap& operator=(const DeviceHeap&) = delete;
    ~DeviceHeap();
    cudaError_t Alloc(size_t bytes, void** out);
    // The caller has finished every use of the block (its stream drained).
    void Free(void* p);
    // Reusable once the work queued on `stream` so far has completed.
    cudaError_t FreeAfter(void* p, cudaStream_t stream);
    // While held (live servers), empty slabs stay mapped for restores.
    void Hold(bool hold);
    size_t Reserved() const;
    size_t InUse() const;

  private:
    struct Slab {
        char* base = nullptr;
        size_t bytes = 0;
    };
    struct FreeRange {
        size_t bytes;
        int slab;
    };
    struct LiveBlock {
        size_t bytes;
        int slab;
    };
    struct Pending {
        char* p;
        cudaEvent_t done;
    };
    void InsertFree(char* p, size_t bytes, int slab);
    void EraseSized(char* p, size_t bytes);
    void Reclaim(bool wait);
    void ReleaseBlock(char* p);
    void TrimEmptySlabs();

    mutable std::mutex mu_;
    std::vector<Slab> slabs_;
    std::map<char*, FreeRange> free_;           // by address: coalescing
    std::multimap<size_t, char*> bySize_;       // by size: best fit
    std::unordered_map<char*, LiveBlock> live_;
    std::deque<Pending> pending_;
    std::vector<cudaEvent_t> spareEvents_;
    size_t reserved_ = 0, inUse_ = 0;
    int holds_ = 0;
};

StepParams MakeParams(const bepugpu_settings& s, float dt);

// An NVTX range for the duration of a scope: the host-side phases (steps,
// batched calls, waves, uploads, downloads) show up by name in Nsight traces.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Island groups (groups.cu).  A group is a set of whole islands run by one CTA.
struct GroupDesc {
    int32_t mBegin, mEnd;   // manifold slots
    int32_t bBegin, bEnd;   // entries of the group body list
    int32_t cBegin, cCount; // colour offsets (relative to mBegin) in the offsets table
    int32_t jBegin, jEnd;   // joint slots
    int32_t jcBegin;        // joint colour offsets (relative to jBegin), cCount + 1 entries
    int32_t pad0, pad1, pad2;
};
struct GroupTables {
    const GroupDesc* groups;
    const int32_t* bodies;        // global indices of each group's dynamic bodies
    const int2* refs;             // per manifold slot: body refs inside the group kernel
    const int32_t* colourOffsets;
    const int2* jointRefs;        // per joint slot: body refs (-1 = the world entity)
    const int32_t* jointColourOffsets;
};
struct GroupPolicy {
    bool enabled = true;
    int32_t maxGroupBodies = 1024;       // shared memory: 96 bytes per body
    int32_t maxGroupManifolds = 4096;    // larger islands stay on the sweep path
    int32_t targetGroupManifolds = 64;   // small islands are packed up to this size
    uint32_t sharedLanesBudget = 200 * 1024;  // groups needing more keep their lanes in global memory
};
// Groups [begin, end) of one kernel variant and the sizes its launch needs.
struct GroupClass {
    int32_t begin = 0, end = 0, maxLocal = 0, maxManifolds = 0, maxColourMembers = 0, maxJoints = 0;
};
struct GroupPlan {
    // groups in launch order: without joints (manifold lanes in shared memory,
    // then in global memory), then with joints (the same two kinds); each kind
    // is one launch sized for its own largest group
    std::vector<GroupDesc> groups;
    std::vector<int32_t> groupBodies, localOf, groupOfManifold, slotOf, globalOffsets, colourOffsets;
    std::vector<int2> refs;  // per slot
    int32_t globalCount = 0;
    GroupClass shared, global, sharedJoints, globalJoints;
    // joints: slots (sweep part first, then the groups'), sweep colour offsets,
    // group colour offsets and refs per slot
    std::vector<int32_t> jointSlotOf, jointGlobalOffsets, jointColourOffsets;
    std::vector<int2> jointRefs;
    int32_t jointGlobalCount = 0;
    bool groupJoints = false;  // some group holds joints
    bool nonConvexLanes = false;  // some group holds a NONCONVEX manifold: shared lanes have room for its friction
};
// Shared memory a group may use: 96 bytes per body, plus 400 per manifold when
// its solve lanes live there.
constexpr size_t kGroupSmemBudget = 200 * 1024;
void PlanGroups(const GroupPolicy& pol, const int32_t* a, const int32_t* b, const int32_t* colour, int32_t nj,
                int32_t nm, const uint8_t* dynamic, int32_t nb, int32_t colours, GroupPlan& plan,
                const uint8_t* nonConvex = nullptr, const int32_t* entryKind = nullptr,
                const uint8_t* follows = nullptr);
// Launches a step of every island group (launches: incremented per kernel
// launch).  With the split prologue (SplitGroupPrologue) two grid-wide
// launches run the groups' refresh, body updates and prestep first.
bepugpu_status LaunchGroups(Context* ctx, Scene* s, const StepParams& p, uint32_t flags, bool count,
                            int* launches = nullptr);
bool SplitGroupPrologue(const Scene* s, uint32_t flags);
// The split prologue's default: scenes whose groups hold joints and at least
// this many constraints.  Measured on GB300: joint chains (151,073 bodies,
// 196,608 joints) step 7 % faster split, 12 % with the added joint types;
// contact-only groups (the 65,536-box pile, towers) 7-13 % slower, the group
// CTA's own pass over its bodies and manifolds being cheaper there than two
// more launches and the copy of the solve lanes.
constexpr int32_t kSplitPrologueConstraints = 8192;
// Joints (joints.cu): record checks, upload into the scene's joint slots, and
// the accumulated impulses back into records.
bepugpu_status CheckJointRecords(Context* ctx, const bepugpu_joint* joints, uint32_t nj, int32_t bodies);
bepugpu_status UploadJoints(Context* ctx, Scene* s, const bepugpu_joint* joints, uint32_t nj);
bepugpu_status DownloadJoints(Context* ctx, Scene* s, bepugpu_joint* joints, uint32_t nj);
// Damping flags bit 2 marks a body stepped by a group kernel.
constexpr uint32_t kOwnedByGroup = 4u;

// The host's account of a scene's kinematic bodies, from the records it
// uploaded and the stages it has run since: whether their candidacy and
// position stages change anything.  A kinematic body's velocity does not
// change on the device, so its stages follow from its record.  A "still"
// body (zero velocity, not always active) settles within two candidacy
// updates: velocity_time_below_limit < 0 becomes 0, 0 becomes 1, and from then
// on the body is inactive and its stages leave it as it is
// (SimulationIslandMember.cs:102-122).
struct KinematicState {
    bool live = false;   // a kinematic body moves or is always active: stages every step
    bool neg = false;    // a still body with velocity_time_below_limit < 0
    bool zero = false;   // a still body with velocity_time_below_limit == 0
    bool prev = false;   // a still, inactive body whose previous_velocity is not yet 0
    void Clear() { live = neg = zero = prev = false; }
    // Adds one kinematic body from its record fields.
    __host__ __device__ void Add(bool moving, uint32_t activity, float previousVelocity, float timeBelowLimit) {
        if (moving || (activity & BEPUGPU_BODY_ALWAYS_ACTIVE)) live = true;
        else if (timeBelowLimit < 0.f) neg = true;
        else if (timeBelowLimit == 0.f) zero = true;
        else if (previousVelocity != 0.f) prev = true;
    }
    // Whether a step with `flags` changes a kinematic body.
    bool Needed(uint32_t flags) const {
        if (live) return (flags & (BEPUGPU_STEP_DEACTIVATION | BEPUGPU_STEP_POSITIONS)) != 0;
        return ((flags & BEPUGPU_STEP_DEACTIVATION) && (neg || zero || prev)) ||
               ((flags & BEPUGPU_STEP_POSITIONS) && (neg || zero));
    }
    // The state after a step with `flags`.
    void Advance(uint32_t flags) {
        if (flags & BEPUGPU_STEP_DEACTIVATION) {
            zero = neg;
            neg = false;
            prev = false;
        }
    }
    // Record-check word bits (k_check_body_records) and back.
    __host__ __device__ uint32_t Bits() const { return (live ? 1u : 0u) | (neg ? 2u : 0u) | (zero ? 4u : 0u) | (prev ? 8u : 0u); }
    void FromBits(uint32_t b) { live = b & 1u; neg = b & 2u; zero = b & 4u; prev = b & 8u; }
};

// Layout of a scene's device scratch block (kScratchBytes): grid barrier
// arrival counter, barrier generation, error word, record-check words, census
// accumulators, timer stamps -- each on its own 128-byte line.
constexpr size_t kScratchBytes = 1024;
constexpr size_t kBarrierCounterAt = 0, kBarrierGenerationAt = 128, kErrorAt = 256, kCheckAt = 384, kCensusAt = 512,
                 kStampsAt = 640;

// Byte offsets of a scene's device arrays inside its arena.
struct ArenaLayout {
    size_t pos, quat, vlin, vang, inv0, inv1, loc0, loc1, damp, m33, act, rawDamp;
    size_t head, cpos, cnrm, offA, offB, mat, pen, fric, axis, pj0, pj1, pj2, s0, s1, s3, s4, s5, s6, s7, lev,
        cfr, cfa, cfb, state, slot, offs;
    size_t jhead, jlanes, jstate, joffs;
    size_t groups, groupBodies, groupRefs, groupOffsets, sweepBodies;
    size_t groupJointRefs, groupJointOffsets;
    size_t bodyRecords;
    size_t shape, genSlots;
};

struct Server;

struct Scene {
    int32_t id = 0;
    Server* server = nullptr;     // a server owns the scene's residency and steps (serve.cu)
    unsigned int* BarrierCounter() const { return (unsigned int*)((char*)counter + kBarrierCounterAt); }
    unsigned int* BarrierGeneration() const { return (unsigned int*)((char*)counter + kBarrierGenerationAt); }
    int* ErrorWord() const { return (int*)((char*)counter + kErrorAt); }
    unsigned long long* Census() const { return (unsigned long long*)((char*)counter + kCensusAt); }
    int* CheckWords() const { return (int*)((char*)counter + kCheckAt); }  // record checks of update calls
    unsigned long long* Stamps() const { return (unsigned long long*)((char*)counter + kStampsAt); }
    int persistentBlocksPerSm = 1;
    int32_t maxBodyReferenced = -1;
    GroupPolicy policy;
    GroupPlan groupPlan;
    GroupDesc* groupDescDev = nullptr;
    int32_t* groupBodiesDev = nullptr;
    int2* groupRefsDev = nullptr;
    int32_t* groupColourOffsetsDev = nullptr;
    int2* groupJointRefsDev = nullptr;
    int32_t* groupJointColourOffsetsDev = nullptr;
    std::vector<uint8_t> hostOwned;  // body stepped by a group kernel
    int32_t* sweepBodiesDev = nullptr;  // bodies no group steps (valid when groups exist)
    uint32_t sweepBodyCount = 0;
    uint32_t sweepDynamicCount = 0;     // dynamic bodies among them
    KinematicState kin;                 // what the kinematic bodies' stages still have to do
    bool asyncPending = false;          // a one-scene step may still run on `stream`
    // Nothing is left for the colour-sweep path: every constraint and dynamic
    // body is in an island group.  (Kinematic bodies may still need their
    // stages: KinematicState.)
    bool SweepEmpty() const {
        return !groupPlan.groups.empty() && groupPlan.globalCount == 0 && groupPlan.jointGlobalCount == 0 &&
               sweepDynamicCount == 0;
    }
    // The whole step of `flags` is island groups without joints or
    // narrow-phase manifolds, and no kinematic body has a stage to run, so a
    // batched launch can run it (batch.cu).
    bool BatchReady(uint32_t flags) const;
    // Narrow phase (collide.cu): one shape per body once uploaded, and the
    // slots of GENERATED manifolds.
    std::vector<bepugpu_shape> hostShapes;
    float4* shape = nullptr;           // device: size xyz, type bits in w
    int32_t* genSlotsDev = nullptr;    // device: slots of GENERATED manifolds, ascending
    int32_t generatedCount = 0;
    std::vector<int2> hostGenPairs;    // bodies of each GENERATED manifold
    // The colour-sweep part of the joint list: slots [0, jointGlobalCount).
    JointSoA SweepJoints() const {
        JointSoA s = j;
        s.count = groupPlan.jointGlobalCount;
        return s;
    }
    int groupThreadsOverride = 0;    // 0 = derived from the plan
    int groupPrologue = -1;          // split group prologue: 1 on, 0 off, -1 by size (SplitGroupPrologue)
    bool phaseEvents = true;         // the step graph records the sweep-path phase events
    bool planStale = false;          // dynamic flags changed since the constraints were planned
    uint64_t batchStamp = 0;         // last batched call listing the scene (duplicate check)
    cudaEvent_t evGroup[2] = {nullptr, nullptr};
    bepugpu_status UploadGroups(Context* ctx);
    bepugpu_status RebuildSweepBodies(Context* ctx);
    // The colour-sweep part of the manifold list: slots [0, globalCount).
    ManifoldSoA SweepManifolds() const {
        ManifoldSoA g = m;
        g.count = groupPlan.globalCount;
        return g;
    }
    int SweepColours() const { return manifoldOffsets.empty() ? 0 : (int)manifoldOffsets.size() - 1; }
    uint32_t maxBodies = 0, maxManifolds = 0, maxJoints = 0;
    DeviceHeap* heap = nullptr;     // the owning context's heap: arena and staging blocks
    void* arena = nullptr;          // null while spilled
    size_t arenaBytes = 0;
    ArenaLayout layout{};
    void* spillHost = nullptr;      // pinned copy of the arena while spilled
    bool spillHostBorrowed = false; // spillHost belongs to a server's pinned pool
    cudaEvent_t evSpill = nullptr, evRestore = nullptr;
    void Rebase();
    bepugpu_status Spill(Context* ctx, bool wait = true, void* host = nullptr);
    bepugpu_status Restore(Context* ctx, cudaStream_t q = nullptr, bool wait = true);
    void DropBorrowedSpillBuffer();
    bool OwnSpillBuffer();
    // Lends a pinned buffer of arenaBytes for spills (kept until dropped);
    // false if the scene already has one.
    bool LendSpillBuffer(void* host) {
        if (spillHost || !host) return false;
        spillHost = host;
        spillHostBorrowed = true;
        return true;
    }
    size_t DeviceBytes() const { return arenaBytes + stagingBytes; }
    void* staging = nullptr;
    size_t stagingBytes = 0;
    size_t stagingManifoldsAt = 0;  // manifold records start here in staging (body records first)
    void* counter = nullptr;  // grid barrier counter / generation / error word
    BodySoA b{};
    ManifoldSoA m{};
    float* localM33 = nullptr;
    int32_t* slotOf = nullptr;           // device: manifold record -> slot
    int32_t* colourOffsetsDev = nullptr; // device: manifold slot range per colour
    uint32_t jointCount = 0;
    bool addedJointTypes = false;         // a joint of type 6 or above: kernels with every joint branch
    JointSoA j{};                         // joint slots in colour order (joints.cu)
    std::vector<int32_t> jointOffsets;    // joint slot range per sweep colour
    std::vector<int32_t> hostJointSlotOf; // joint record -> slot
    int32_t* jointOffsetsDev = nullptr;
    bepugpu_body* bodyRecords = nullptr;  // device copy of the last uploaded body records (downloads patch it)
    std::vector<float4> hostJointAcc;     // download scratch: [2][joints]
    Colouring colouring;
    std::vector<int32_t> manifoldOffsets;
    std::vector<int32_t> hostSlotOf;
    std::vector<float> hostLinDamp, hostAngDamp, hostLocalM33;
    std::vector<float2> hostRawDamp;
    std::vector<uint8_t> hostDynamic;
    std::vector<int32_t> hostKinematic;  // indices of the bodies uploaded with is_dynamic = 0
    std::vector<float4> hostDamp;
    bool dampDirty = true;
    float dampDt = 0.f;
    cudaStream_t stream = nullptr;
    cudaEvent_t evStart = nullptr, evStop = nullptr;
    cudaEvent_t evPhase[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    bool stepped = false;
    int32_t mode = BEPUGPU_MODE_GRAPH;
    cudaGraphExec_t graphExec = nullptr;
    float graphDt = 0.f;
    uint32_t graphFlags = 0;
    uint64_t version = 1, graphVersion = 0;
    bool graphTail = false;  // the graph ends with the kinematic bodies' stages
    bool graphWakes = false; // the graph's island stage looks for kinematic wakes
    int graphIterations = -1;
    uint32_t launchesPerStep = 0;
    int persistentBlocks = 0;
    bool persistentAdded = false;  // the persistent variant persistentBlocks was sized for
    BroadPhaseBuffers* broadPhase = nullptr;  // device buffers of bepugpu_broad_phase (broadphase.cu)
    IslandBuffers* islands = nullptr;         // bepugpu_set_islands (islands.cu); null: every island awake
    PairBuffers* pairs = nullptr;             // bepugpu_update_pairs (pairs.cu): materials and scratch
    // With islands the deactivation stage runs first, in its own launches
    // (LaunchIslandStage); the other stages then run without it.
    uint32_t StageFlags(uint32_t flags) const {
        return islands ? flags & ~(uint32_t)BEPUGPU_STEP_DEACTIVATION : flags;
    }

    ~Scene();
    bepugpu_status Allocate(Context* ctx, uint32_t nb, uint32_t nm, uint32_t nj);
    bepugpu_status RefreshDamping(Context* ctx, float dt);
    bepugpu_status BuildGraph(Context* ctx, const StepParams& p, uint32_t flags);
    bepugpu_status RunPersistent(Context* ctx, const StepParams& p, uint32_t flags);
    bepugpu_status Step(Context* ctx, float dt, uint32_t flags);
};

struct BatchEngine {
    virtual ~BatchEngine() = default;
};

// A scene's island state for batched launches (islands.cu; n = 0 without islands).
struct IslandView {
    uint32_t* flags;
    const int32_t* members;
    int32_t* candidates;
    int32_t* wakeAt;
    int32_t* index;
    unsigned int* done;
    int n;
};
void FillIslandView(const Scene& s, IslandView& v);

// Batched launches (batch.cu): one CTA per work item {view, group, steps}.
struct SceneView {
    ManifoldSoA m;
    BodySoA b;
    GroupTables t;
    IslandView isl;
};
SceneView MakeView(const Scene& s);
cudaError_t LaunchBatchedGroups(bool shared, const SceneView* views, const int4* work, int n, const StepParams& p,
                                uint32_t flags, int Bc, int Lc, int members, int threads, int passes,
                                cudaStream_t stream, bool nonConvex = false, int firstPass = 0);
// The island stage of the batched scenes with islands (islands.cu): work items
// {view, body block of 256, the scene's blocks, steps}, for step `pass`.
cudaError_t LaunchBatchedIslands(const SceneView* views, const int4* work, int n, const StepParams& p,
                                 int maxAttempts, int pass, cudaStream_t stream);
// Work items of LaunchBatchedIslands for view `vi` of scene s stepping `steps` times.
void AddIslandWork(const Scene& s, int vi, int steps, std::vector<int4>& work);

struct Context {
    int device = 0;
    int smCount = 0;
    bepugpu_settings settings{};
    std::string lastError;
    std::unique_ptr<DeviceHeap> heap;  // declared before the scenes: it outlives them
    std::unordered_map<int32_t, std::unique_ptr<Scene>> scenes;
    int32_t nextScene = 1;
    std::unique_ptr<BatchEngine> batch;
    uint32_t lastLaunches = 0;
    float lastMs = 0.f;
    int batchThreads = 0;  // threads per CTA of batched launches, 0 = from the groups' colour sizes
    uint64_t batchEpoch = 0;  // batched calls so far (Scene::batchStamp)
    std::vector<bepugpu_server*> servers;  // live servers: shut down before the scenes go
    void SetError(const char* fmt, ...);
};

// A scene of the context that no server owns (null and an error message
// otherwise), and the status for a missing one: NOT_FOUND, or
// INVALID_OPERATION when a server owns it.
Scene* FindScene(Context* ctx, int32_t id);
bepugpu_status SceneMissing(Context* ctx, int32_t id);

// Narrow phase (collide.cu).  Checks the GENERATED manifolds of a constraint
// upload against the scene's shapes and their contact_order fields, and
// stores their slots; LaunchCollide runs the narrow phase over them.
bepugpu_status PrepareGenerated(Context* ctx, Scene* s, const bepugpu_manifold* man, uint32_t nm,
                                const std::vector<int32_t>& slotOf);
cudaError_t LaunchCollide(Scene* s, const StepParams& p, cudaStream_t stream);

// Stops every server of the context and gives its scenes back; their handles
// then accept only bepugpu_server_destroy (serve.cu).
void ShutdownServers(Context* ctx);

}  // namespace bepugpu
