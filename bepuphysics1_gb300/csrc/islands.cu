// Simulation islands on the device: DeactivationManager.Update without the
// split flush (DeactivationManagement/DeactivationManager.cs:216-224,310-336)
// over the island partition and list order the host keeps.
//
// The reference's candidacy loop runs member by member; the only coupling
// between members is an active kinematic member waking its connections'
// islands (SimulationIslandMember.cs:135-159), which decides whether a later
// member of such an island is updated as active.  Two launches restate the
// loop: every connection of an active kinematic body records, per island, the
// lowest member index that wakes it (k_island_wakes, only while a kinematic
// body can wake anything); every member then runs its candidacy update with
// its island's state at its own turn -- awake from the start, or woken by a
// member before it -- and counts the island's candidates, and the launch's
// last block applies the wakes and runs DeactivateObjects' round robin
// (k_island_members).
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "joints_device.cuh"
#include "scan_device.cuh"
#include "solver_device.cuh"

namespace bepugpu {

// Device state of a scene's islands: one block of cudaMalloc memory.
struct IslandBuffers {
    int32_t n = 0, nb = 0;
    void* block = nullptr;
    int32_t* islandOf = nullptr;   // [nb] island of each body, -1 kinematic
    uint32_t* flags = nullptr;     // [n] BEPUGPU_ISLAND_*
    int32_t* members = nullptr;    // [n] SimulationIsland.memberCount
    int32_t* candidates = nullptr; // [n] members that are deactivation candidates (scratch, zero between steps)
    int32_t* wakeAt = nullptr;     // [n] lowest waking kinematic member (scratch, INT_MAX between steps)
    int32_t* index = nullptr;      // [1] deactivationIslandIndex
    unsigned int* done = nullptr;  // [1] blocks of k_island_members finished (zero between steps)
    ~IslandBuffers() { cudaFree(block); }
};

namespace {

// The kinematic body a constraint connects to an island, or -1.
__device__ __forceinline__ void WakeThrough(const BodySoA& b, int k, int other, const StepParams& p,
                                            int32_t* wakeAt) {
    if (k < 0 || other < 0 || b.pos[k].w != 0.f) return;  // k must be a kinematic body
    const int island = b.islandOf[other];
    if (island < 0) return;  // two kinematic bodies
    float4 act = b.act[k];
    if (!(act.y <= 0.f)) return;  // inactive at its turn: no update, no wake (:61-62)
    CandidacyMath(b.vlin[k], b.vang[k], false, act, p);
    if (act.y <= 0.f) atomicMin(wakeAt + island, k);
}

// Connections of kinematic bodies: every joint slot and every manifold slot
// with contacts (a pair handler's constraint is in the solver only then).
__global__ void k_island_wakes(ManifoldSoA m, JointSoA j, BodySoA b, StepParams p, int32_t* wakeAt) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int4 h;
    if (t < m.count) {
        h = m.head[t];
        if ((h.z & 0xff) == 0) return;
    } else if (t - m.count < j.count) {
        h = j.head[t - m.count];
    } else {
        return;
    }
    WakeThrough(b, h.x, h.y, p, wakeAt);
    WakeThrough(b, h.y, h.x, p, wakeAt);
}

// The wakes (island.IsActive = true, allowDeactivation = false), then
// DeactivateObjects (DeactivationManager.cs:310-336) with TryToDeactivate
// (SimulationIsland.cs:94-118), then the scratch cleared; by one block.  The
// round robin looks at a run of islands after the index, each while the
// members of the run's islands before it add up to less than the budget and
// the run is shorter than the list; TryToDeactivate of one island reads only
// that island, so the run is decided a block-wide chunk at a time from a
// prefix sum of member counts.  The counts other blocks added are read from L2.
__device__ void DeactivateObjects(uint32_t* flags, const int32_t* __restrict__ members, int32_t* candidates,
                                  int32_t* wakeAt, int32_t* index, int n, int maxAttempts, bool wakes) {
    __shared__ int warpSums[32];
    __shared__ int lastLooked, counted;
    if (wakes) {  // eight loads in flight a thread, then their islands
        constexpr int kBatch = 8;
        for (int k0 = threadIdx.x; k0 < n; k0 += kBatch * blockDim.x) {
            int w[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
                const int k = k0 + u * (int)blockDim.x;
                w[u] = k < n ? __ldcg(wakeAt + k) : INT_MAX;
            }
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
                const int k = k0 + u * (int)blockDim.x;
                if (w[u] != INT_MAX) {
                    flags[k] = (flags[k] | BEPUGPU_ISLAND_ACTIVE) & ~BEPUGPU_ISLAND_ALLOW_DEACTIVATION;
                    wakeAt[k] = INT_MAX;
                }
            }
        }
    }
    if (threadIdx.x == 0) {
        lastLooked = -1;
        counted = 0;
    }
    __syncthreads();
    const int start = *index;
    for (int base = 0; base < n; base += blockDim.x) {
        const int k = base + (int)threadIdx.x;  // position in the run
        const int island = (start + 1 + k) % n;
        const int m = k < n ? members[island] : 0;
        const int before = counted;  // members of the run before this chunk
        const int incl = BlockInclusiveSum(m, warpSums);
        const bool looked = k < n && before + (incl - m) < maxAttempts;
        if (looked) {
            uint32_t f = flags[island];
            if (f & BEPUGPU_ISLAND_ALLOW_DEACTIVATION) {
                if ((f & BEPUGPU_ISLAND_ACTIVE) && __ldcg(candidates + island) == m) f &= ~BEPUGPU_ISLAND_ACTIVE;
            } else {
                f |= BEPUGPU_ISLAND_ALLOW_DEACTIVATION;
            }
            flags[island] = f;
            atomicMax(&lastLooked, k);
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) counted = before + incl;
        __syncthreads();
        if (counted >= maxAttempts || lastLooked < base + (int)blockDim.x - 1) break;
    }
    if (threadIdx.x == 0 && lastLooked >= 0) *index = (start + 1 + lastLooked) % n;
    __syncthreads();
    for (int k = threadIdx.x; k < n; k += blockDim.x) candidates[k] = 0;
}

// UpdateDeactivationCandidacy of every member (SimulationIslandMember.cs:53-164);
// the last block to finish then runs DeactivateObjects.
__global__ void k_island_members(BodySoA b, StepParams p, int32_t* wakeAt, int32_t* candidates, uint32_t* flags,
                                 const int32_t* __restrict__ members, int32_t* index, int n, int maxAttempts,
                                 unsigned int* done, bool wakes) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < b.count) {
        const bool dynamic = b.pos[i].w != 0.f;
        float4 act = b.act[i];
        if (dynamic) {
            const int island = b.islandOf[i];
            const bool awake = (b.islandFlags[island] & BEPUGPU_ISLAND_ACTIVE) || (wakes && wakeAt[island] < i);
            CandidacyMath(b.vlin[i], b.vang[i], true, act, p, awake);
            if (__float_as_uint(act.z) & kCandidate) atomicAdd(candidates + island, 1);
        } else {
            CandidacyMath(b.vlin[i], b.vang[i], false, act, p);
        }
        b.act[i] = act;
    }
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    DeactivateObjects(flags, members, candidates, wakeAt, index, n, maxAttempts, wakes);
    if (threadIdx.x == 0) *done = 0u;
}

// The island stage of batched scenes: a block per work item {view, body block,
// the scene's blocks, steps}; the last block of a scene runs its
// DeactivateObjects (batched scenes have no kinematic body that can wake an island).
__global__ void k_batch_island_members(const SceneView* __restrict__ views, const int4* __restrict__ work,
                                       StepParams p, int maxAttempts, int pass) {
    const int4 w = work[blockIdx.x];
    if (pass >= w.w) return;
    const SceneView& v = views[w.x];
    const BodySoA b = v.b;
    const int i = w.y * blockDim.x + threadIdx.x;
    if (i < b.count) {
        const bool dynamic = b.pos[i].w != 0.f;
        float4 act = b.act[i];
        if (dynamic) {
            const int island = b.islandOf[i];
            CandidacyMath(b.vlin[i], b.vang[i], true, act, p, (b.islandFlags[island] & BEPUGPU_ISLAND_ACTIVE) != 0);
            if (__float_as_uint(act.z) & kCandidate) atomicAdd(v.isl.candidates + island, 1);
        } else {
            CandidacyMath(b.vlin[i], b.vang[i], false, act, p);
        }
        b.act[i] = act;
    }
    __shared__ bool last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(v.isl.done, 1u) == (unsigned)w.z - 1;
    __syncthreads();
    if (!last) return;
    __threadfence();
    DeactivateObjects(v.isl.flags, v.isl.members, v.isl.candidates, v.isl.wakeAt, v.isl.index, v.isl.n, maxAttempts,
                      false);
    if (threadIdx.x == 0) *v.isl.done = 0u;
}

// Every joint and every manifold with contacts keeps its dynamic bodies in
// one island; *bad receives the lowest slot (joints after manifolds) that does not.
__global__ void k_check_islands(ManifoldSoA m, JointSoA j, BodySoA b, int* bad) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int4 h;
    if (t < m.count) {
        h = m.head[t];
        if ((h.z & 0xff) == 0) return;
    } else if (t - m.count < j.count) {
        h = j.head[t - m.count];
    } else {
        return;
    }
    const int ia = h.x >= 0 ? b.islandOf[h.x] : -1, ib = h.y >= 0 ? b.islandOf[h.y] : -1;
    if (ia >= 0 && ib >= 0 && ia != ib) atomicMin(bad, t);
}

}  // namespace

#define CK(call)                                                                              \
    do {                                                                                      \
        cudaError_t e_ = (call);                                                              \
        if (e_ != cudaSuccess) {                                                              \
            ctx->SetError("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
            return BEPUGPU_CUDA_ERROR;                                                        \
        }                                                                                     \
    } while (0)

void ReleaseIslands(Scene* s) {
    delete s->islands;
    s->islands = nullptr;
    s->b.islandOf = nullptr;
    s->b.islandFlags = nullptr;
}

void ApplyIslandViews(Scene* s) {
    s->b.islandOf = s->islands ? s->islands->islandOf : nullptr;
    s->b.islandFlags = s->islands ? s->islands->flags : nullptr;
}

void FillIslandView(const Scene& s, IslandView& v) {
    const IslandBuffers* I = s.islands;
    v.flags = I ? I->flags : nullptr;
    v.members = I ? I->members : nullptr;
    v.candidates = I ? I->candidates : nullptr;
    v.wakeAt = I ? I->wakeAt : nullptr;
    v.index = I ? I->index : nullptr;
    v.done = I ? I->done : nullptr;
    v.n = I ? I->n : 0;
}

void AddIslandWork(const Scene& s, int vi, int steps, std::vector<int4>& work) {
    if (!s.islands) return;
    const int blocks = std::max(1, (s.b.count + 255) / 256);
    for (int k = 0; k < blocks; k++) work.push_back(make_int4(vi, k, blocks, steps));
}

cudaError_t LaunchBatchedIslands(const SceneView* views, const int4* work, int n, const StepParams& p,
                                 int maxAttempts, int pass, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    k_batch_island_members<<<(unsigned)n, 256, 0, stream>>>(views, work, p, maxAttempts, pass);
    return cudaGetLastError();
}

// Kinematic members can wake islands in this step: one moves or is always
// active (its update leaves its time flag at -1), or a still one's flag is
// below 0 (the update takes it to 0).
bool IslandWakesPossible(const Scene* s) {
    return !s->hostKinematic.empty() && (s->kin.live || s->kin.neg);
}

cudaError_t LaunchIslandStage(Scene* s, const StepParams& p, int maxAttempts, cudaStream_t q) {
    IslandBuffers& I = *s->islands;
    const int T = 128;
    const int nc = s->m.count + s->j.count;
    const bool wakes = IslandWakesPossible(s) && nc > 0;  // else every wakeAt stays INT_MAX
    if (wakes) {
        k_island_wakes<<<(nc + T - 1) / T, T, 0, q>>>(s->m, s->j, s->b, p, I.wakeAt);
        s->launchesPerStep++;
    }
    // at least one block: its last one runs DeactivateObjects
    const int blocks = std::max(1, (s->b.count + 255) / 256);
    k_island_members<<<blocks, 256, 0, q>>>(s->b, p, I.wakeAt, I.candidates, I.flags, I.members, I.index, I.n,
                                            maxAttempts, I.done, wakes);
    s->launchesPerStep++;
    return cudaGetLastError();
}

}  // namespace bepugpu

using namespace bepugpu;

extern "C" bepugpu_status bepugpu_set_islands(bepugpu_context* c, int32_t id, const int32_t* island_of_body,
                                              uint32_t body_count, const uint32_t* island_flags, uint32_t islands,
                                              int32_t deactivation_index) {
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    if (s->asyncPending) {
        CK(cudaStreamSynchronize(s->stream));
        s->asyncPending = false;
    }
    if (islands == 0) {
        ReleaseIslands(s);
        s->version++;
        return BEPUGPU_OK;
    }
    const int32_t nb = s->b.count;
    if (body_count != (uint32_t)nb || !island_of_body || !island_flags) {
        ctx->SetError("set_islands: one island index for each of the %d bodies and one flag word per island", nb);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (deactivation_index < 0 || (uint32_t)deactivation_index >= islands) {
        ctx->SetError("set_islands: deactivation_index %d outside [0, %u)", deactivation_index, islands);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    std::vector<int32_t> members(islands, 0);
    for (int32_t i = 0; i < nb; i++) {
        const int32_t k = island_of_body[i];
        const bool dynamic = (size_t)i < s->hostDynamic.size() && s->hostDynamic[i];
        if (!dynamic) {
            if (k != -1) {
                ctx->SetError("set_islands: kinematic body %d has island %d (kinematic bodies take -1)", i, k);
                return BEPUGPU_INVALID_ARGUMENT;
            }
            continue;
        }
        if (k < 0 || (uint32_t)k >= islands) {
            ctx->SetError("set_islands: dynamic body %d has island %d outside [0, %u)", i, k, islands);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        members[k]++;
    }
    for (uint32_t k = 0; k < islands; k++) {
        if (!members[k]) {
            ctx->SetError("set_islands: island %u has no member", k);
            return BEPUGPU_INVALID_ARGUMENT;
        }
        if (island_flags[k] & ~(BEPUGPU_ISLAND_ACTIVE | BEPUGPU_ISLAND_ALLOW_DEACTIVATION)) {
            ctx->SetError("set_islands: island %u has unknown flag bits 0x%x", k, island_flags[k]);
            return BEPUGPU_INVALID_ARGUMENT;
        }
    }
    auto* I = new IslandBuffers();
    I->n = (int32_t)islands;
    I->nb = nb;
    const size_t bytes = 4 * ((size_t)nb + 5 * (size_t)islands + 2);
    cudaError_t e = cudaMalloc(&I->block, bytes);
    if (e != cudaSuccess) {
        delete I;
        ctx->SetError("set_islands: %zu bytes: %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? BEPUGPU_OUT_OF_MEMORY : BEPUGPU_CUDA_ERROR;
    }
    auto* w = (int32_t*)I->block;
    I->islandOf = w;
    I->flags = (uint32_t*)(w + nb);
    I->members = w + nb + islands;
    I->candidates = w + nb + 2 * (size_t)islands;
    I->wakeAt = w + nb + 3 * (size_t)islands;
    I->index = w + nb + 4 * (size_t)islands;
    I->done = (unsigned int*)(I->index + 1);
    std::vector<int32_t> wake(islands, INT_MAX);
    auto fail = [&](cudaError_t err) {
        delete I;
        ctx->SetError("set_islands: %s", cudaGetErrorString(err));
        return BEPUGPU_CUDA_ERROR;
    };
    if ((e = cudaMemcpyAsync(I->islandOf, island_of_body, 4 * (size_t)nb, cudaMemcpyHostToDevice, s->stream)) ||
        (e = cudaMemcpyAsync(I->flags, island_flags, 4 * (size_t)islands, cudaMemcpyHostToDevice, s->stream)) ||
        (e = cudaMemcpyAsync(I->members, members.data(), 4 * (size_t)islands, cudaMemcpyHostToDevice, s->stream)) ||
        (e = cudaMemsetAsync(I->candidates, 0, 4 * (size_t)islands, s->stream)) ||
        (e = cudaMemcpyAsync(I->wakeAt, wake.data(), 4 * (size_t)islands, cudaMemcpyHostToDevice, s->stream)) ||
        (e = cudaMemcpyAsync(I->index, &deactivation_index, 4, cudaMemcpyHostToDevice, s->stream)) ||
        (e = cudaMemsetAsync(I->done, 0, 4, s->stream)))
        return fail(e);
    // every connection inside one island, checked against the scene's current contacts
    BodySoA bv = s->b;
    bv.islandOf = I->islandOf;
    bv.islandFlags = I->flags;
    const int nc = s->m.count + s->j.count;
    int bad = INT_MAX;
    if (nc > 0) {
        int* word = s->CheckWords();
        if ((e = cudaMemsetAsync(word, 0x7f, sizeof(int), s->stream))) return fail(e);
        k_check_islands<<<(nc + 127) / 128, 128, 0, s->stream>>>(s->m, s->j, bv, word);
        if ((e = cudaGetLastError()) || (e = cudaMemcpyAsync(&bad, word, sizeof(int), cudaMemcpyDeviceToHost,
                                                             s->stream)))
            return fail(e);
    }
    if ((e = cudaStreamSynchronize(s->stream))) return fail(e);
    if (bad != 0x7f7f7f7f && bad != INT_MAX) {
        delete I;
        if (bad < s->m.count) ctx->SetError("set_islands: manifold slot %d connects two islands", bad);
        else ctx->SetError("set_islands: joint slot %d connects two islands", bad - s->m.count);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    ReleaseIslands(s);
    s->islands = I;
    ApplyIslandViews(s);
    s->version++;
    return BEPUGPU_OK;
}

extern "C" bepugpu_status bepugpu_get_islands(bepugpu_context* c, int32_t id, uint32_t* island_flags,
                                              uint32_t islands, int32_t* deactivation_index) {
    auto* ctx = reinterpret_cast<Context*>(c);
    if (!ctx) return BEPUGPU_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    Scene* s = FindScene(ctx, id);
    if (!s) return SceneMissing(ctx, id);
    const uint32_t n = s->islands ? (uint32_t)s->islands->n : 0u;
    if (islands != n || (n && !island_flags)) {
        ctx->SetError("get_islands: the scene has %u islands", n);
        return BEPUGPU_INVALID_ARGUMENT;
    }
    if (!n) {
        if (deactivation_index) *deactivation_index = 0;
        return BEPUGPU_OK;
    }
    int32_t idx = 0;
    CK(cudaMemcpyAsync(island_flags, s->islands->flags, 4 * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(&idx, s->islands->index, 4, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    s->asyncPending = false;
    if (deactivation_index) *deactivation_index = idx;
    return BEPUGPU_OK;
}
