// Island groups: whole steps of small simulation islands inside one CTA.
//
// An island is a set of dynamic bodies connected through constraints
// (kinematic bodies do not connect, as in the reference's simulation islands,
// DeactivationManagement/SimulationIslandMember.cs).  Constraints of different
// islands never share a dynamic body, so the solver's colour-ordered sequence
// restricted to one island is that island's own Gauss-Seidel sequence and
// islands can run in any interleaving.  Islands small enough to keep their
// bodies in shared memory are packed into groups; one CTA runs a group's whole
// step -- refresh, force update, prestep, warm start, every colour sweep of
// every iteration, position update -- with block barriers between sweeps
// instead of grid-wide ones.  When the group's solve lanes (Jacobians,
// friction lanes, impulses, state) fit too, the prestep writes them to shared
// memory and the sweeps never touch global memory for them.  Larger islands
// stay on the colour-sweep path.
#include <cuda_runtime.h>

#include <algorithm>
#include <numeric>
#include <vector>

#include "../../include/bepugpu.h"
#include "bepugpu_internal.h"
#include "groups_device.cuh"
#include "solver_device.cuh"

namespace bepugpu {

template <bool kCensus, bool kShared, int kJoints>
__global__ void k_groups(ManifoldSoA m, BodySoA b, JointSoA j, StepParams p, uint32_t flags, GroupTables t,
                         int groupBase, int Bc, int Lc, int Jc, unsigned long long* census, bool nonConvex,
                         bool prestepped) {
    extern __shared__ float4 smem[];
    const GroupDesc g = t.groups[groupBase + blockIdx.x];
    GroupStep<kCensus, kShared, kJoints>(m, b, j, p, flags, t, g, Bc, Lc, Jc, smem, census, nonConvex, prestepped);
}

// The group step's first stages as grid-wide launches (the split prologue):
// the contact refresh of the groups' manifold slots [s0, s1) beside the
// candidacy and force updates of their bodies (list[0, n)), then the prestep
// of those slots into the global solve lanes.  One thread per manifold or
// body fills the GPU where a group CTA runs its few threads over them in turn;
// the group kernel then copies the lanes into shared memory
// (GroupStep's `prestepped`).  The same device routines as the colour-sweep
// path's k_refresh_force_list and k_prestep.
__global__ void k_group_refresh_force(ManifoldSoA m, BodySoA b, StepParams p, const int32_t* __restrict__ list, int n,
                                      int s0, int s1, uint32_t flags) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x, nm = s1 - s0;
    if (t < nm) {
        if (flags & BEPUGPU_STEP_REFRESH_CONTACTS) RefreshManifold(m, b, s0 + t, p);
    } else if (t - nm < n) {
        if (flags & (BEPUGPU_STEP_FORCES | BEPUGPU_STEP_DEACTIVATION)) StartBodyStep(b, list[t - nm], p, flags);
    }
}
__global__ void k_group_prestep(ManifoldSoA m, BodySoA b, StepParams p, int s0, int s1) {
    const int s = s0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (s < s1) PrestepManifold(m, b, s, p);
}

// ------------------------------------------------------------------ host side --
namespace {
struct UnionFind {
    std::vector<int32_t> parent;
    explicit UnionFind(int n) : parent(n) { std::iota(parent.begin(), parent.end(), 0); }
    int32_t Find(int32_t x) {
        while (parent[x] != x) {
            parent[x] = parent[parent[x]];
            x = parent[x];
        }
        return x;
    }
    void Join(int32_t a, int32_t b) {
        a = Find(a);
        b = Find(b);
        if (a != b) parent[std::max(a, b)] = std::min(a, b);
    }
};
}  // namespace

// Splits the solver list into the colour-sweep part and island groups and
// assigns every manifold and joint its slot.  colour[u] is the solver-list
// colouring (joints first, u < nj).  The sweep part takes manifold slots
// [0, globalCount) and joint slots [0, jointGlobalCount) in colour-major
// order; each group takes a contiguous manifold range and a contiguous joint
// range, each in colour-major order.  When a group holds a NONCONVEX manifold
// (nonConvex[i] != 0; null: none), every group's shared manifold lanes have
// room for contact friction (plan.nonConvexLanes, GroupManifoldLanes).
//
// Inside a colour no two entries share a dynamic body, so their order does not
// change a sweep's result: entries of a colour take their slots sorted by
// entryKind[u] (null: list order), stably, so that a warp's threads run the same
// branch of the joint and manifold code.  follows[u] != 0 keeps a joint's
// continuation records right after it (they share its kind).
void PlanGroups(const GroupPolicy& pol, const int32_t* a, const int32_t* b, const int32_t* colour, int32_t nj,
                int32_t nm, const uint8_t* dynamic, int32_t nb, int32_t colours, GroupPlan& plan,
                const uint8_t* nonConvex, const int32_t* entryKind, const uint8_t* follows) {
    // A colour's entries (ascending) regrouped: units (an entry and the entries
    // that follow it) stably sorted by the unit's kind.
    auto byKind = [&](std::vector<int32_t>& list) {
        if (!entryKind || list.size() < 2) return;
        std::vector<std::pair<int32_t, int32_t>> units;  // (first index in list, length)
        for (int32_t i = 0; i < (int32_t)list.size(); i++) {
            const int32_t u = list[i];
            if (follows && u < nj && follows[u] && !units.empty()) units.back().second++;
            else units.push_back({i, 1});
        }
        std::stable_sort(units.begin(), units.end(), [&](const std::pair<int32_t, int32_t>& x,
                                                         const std::pair<int32_t, int32_t>& y) {
            return entryKind[list[x.first]] < entryKind[list[y.first]];
        });
        std::vector<int32_t> out;
        out.reserve(list.size());
        for (auto& un : units)
            for (int32_t k = 0; k < un.second; k++) out.push_back(list[un.first + k]);
        list.swap(out);
    };
    plan = GroupPlan();
    const int32_t n = nj + nm;
    std::vector<int32_t> groupOf(n, -1);  // per updateable
    std::vector<std::vector<int32_t>> gBodies;
    plan.localOf.assign(nb, -1);
    if (pol.enabled && n > 0) {
        UnionFind uf(nb);
        for (int32_t u = 0; u < n; u++)
            if (a[u] >= 0 && b[u] >= 0 && dynamic[a[u]] && dynamic[b[u]]) uf.Join(a[u], b[u]);
        std::vector<int32_t> idOfRoot(nb, -1), members, bodiesCount, islandOf(n, -1);
        for (int32_t u = 0; u < n; u++) {
            int32_t ea = a[u], eb = b[u];
            int32_t e = ea >= 0 && dynamic[ea] ? ea : (eb >= 0 && dynamic[eb] ? eb : -1);
            if (e < 0) continue;  // no dynamic body: never active, sweep path
            int32_t root = uf.Find(e);
            if (idOfRoot[root] < 0) {
                idOfRoot[root] = (int32_t)members.size();
                members.push_back(0);
                bodiesCount.push_back(0);
            }
            islandOf[u] = idOfRoot[root];
            members[islandOf[u]]++;
        }
        for (int32_t e = 0; e < nb; e++)
            if (dynamic[e] && idOfRoot[uf.Find(e)] >= 0) bodiesCount[idOfRoot[uf.Find(e)]]++;
        // islands too large for one CTA stay on the sweep path
        std::vector<uint8_t> small(members.size());
        // joints keep their solve lanes in shared memory: an island's bodies and
        // joints must fit a CTA's budget
        std::vector<int32_t> jointsOf(members.size(), 0);
        for (int32_t u = 0; u < nj; u++)
            if (islandOf[u] >= 0) jointsOf[islandOf[u]]++;
        auto fitsCta = [&](int64_t bodies, int64_t joints) {
            return GroupSmemBytes(false, (int)bodies, 0, (int)joints) <= kGroupSmemBudget;
        };
        for (size_t k = 0; k < members.size(); k++)
            small[k] = bodiesCount[k] <= pol.maxGroupBodies && members[k] <= pol.maxGroupManifolds &&
                       fitsCta(bodiesCount[k], jointsOf[k]);
        // pack small islands into groups in island order (joints count like manifolds)
        std::vector<int32_t> groupOfIsland(members.size(), -1);
        int32_t gm = 0, gb = 0, gj = 0, groups = 0;
        for (size_t k = 0; k < members.size(); k++) {
            if (!small[k]) continue;
            if (groups == 0 || gm + members[k] > pol.targetGroupManifolds || gb + bodiesCount[k] > pol.maxGroupBodies ||
                !fitsCta(gb + bodiesCount[k], gj + jointsOf[k])) {
                groups++;
                gm = gb = gj = 0;
            }
            groupOfIsland[k] = groups - 1;
            gm += members[k];
            gb += bodiesCount[k];
            gj += jointsOf[k];
        }
        gBodies.resize(groups);
        for (int32_t e = 0; e < nb; e++) {
            if (!dynamic[e]) continue;
            int32_t id = idOfRoot[uf.Find(e)];
            if (id < 0 || groupOfIsland[id] < 0) continue;
            plan.localOf[e] = (int32_t)gBodies[groupOfIsland[id]].size();
            gBodies[groupOfIsland[id]].push_back(e);
        }
        for (int32_t u = 0; u < n; u++)
            if (islandOf[u] >= 0) groupOf[u] = groupOfIsland[islandOf[u]];
    }
    const int32_t G = (int32_t)gBodies.size();
    std::vector<std::vector<int32_t>> mMembers(G), jMembers(G);
    for (int32_t u = 0; u < n; u++)
        if (groupOf[u] >= 0) (u < nj ? jMembers : mMembers)[groupOf[u]].push_back(u);
    // Launch order by kind: no joints before joints, shared-memory manifold
    // lanes before global ones (kind 0..3), stable inside a kind.
    std::vector<int32_t> order(G);
    std::iota(order.begin(), order.end(), 0);
    std::vector<uint8_t> fits(G), kind(G);
    // Shared manifold lanes have room for contact friction when any group
    // holds a NONCONVEX manifold (one layout for all of the scene's groups).
    if (nonConvex)
        for (int32_t gId = 0; gId < G && !plan.nonConvexLanes; gId++)
            for (int32_t u : mMembers[gId]) plan.nonConvexLanes = plan.nonConvexLanes || nonConvex[u - nj];
    for (int32_t gId = 0; gId < G; gId++) {
        fits[gId] = GroupSmemBytes(true, (int)gBodies[gId].size(), (int)mMembers[gId].size(),
                                   (int)jMembers[gId].size(), plan.nonConvexLanes) <=
                    std::min<size_t>(pol.sharedLanesBudget, kGroupSmemBudget);
        kind[gId] = (uint8_t)((jMembers[gId].empty() ? 0 : 2) + (fits[gId] ? 0 : 1));
    }
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return kind[x] < kind[y]; });
    GroupClass* classes[4] = {&plan.shared, &plan.global, &plan.sharedJoints, &plan.globalJoints};

    // Sweep slots, colour-major: manifolds and joints not in a group.
    plan.slotOf.assign(nm, -1);
    plan.jointSlotOf.assign(nj, -1);
    plan.globalOffsets.assign(colours + 1, 0);
    plan.jointGlobalOffsets.assign(colours + 1, 0);
    int32_t slot = 0, jslot = 0;
    {
        std::vector<std::vector<int32_t>> byColour(colours);
        for (int32_t u = 0; u < n; u++)
            if (groupOf[u] < 0) byColour[colour[u]].push_back(u);
        for (int32_t c = 0; c < colours; c++) {
            byKind(byColour[c]);
            plan.globalOffsets[c] = slot;
            plan.jointGlobalOffsets[c] = jslot;
            for (int32_t u : byColour[c]) {
                if (u < nj) plan.jointSlotOf[u] = jslot++;
                else plan.slotOf[u - nj] = slot++;
            }
        }
        plan.globalOffsets[colours] = slot;
        plan.jointGlobalOffsets[colours] = jslot;
        plan.globalCount = slot;
        plan.jointGlobalCount = jslot;
    }
    plan.refs.assign(nm, make_int2(-1, -1));
    plan.jointRefs.assign(nj, make_int2(-1, -1));
    plan.groupOfManifold.assign(nm, -1);
    plan.groups.resize(G);
    auto ref = [&](int32_t e) -> int32_t {
        if (e < 0) return -1;
        return dynamic[e] ? plan.localOf[e] : -2 - e;
    };
    for (int32_t k = 0; k < G; k++) {
        const int32_t gId = order[k];
        GroupDesc& d = plan.groups[k];
        d = GroupDesc{};
        GroupClass& cls = *classes[kind[gId]];
        if (cls.end == cls.begin) cls.begin = cls.end = k;
        cls.end = k + 1;
        d.bBegin = (int32_t)plan.groupBodies.size();
        plan.groupBodies.insert(plan.groupBodies.end(), gBodies[gId].begin(), gBodies[gId].end());
        d.bEnd = (int32_t)plan.groupBodies.size();
        cls.maxLocal = std::max(cls.maxLocal, d.bEnd - d.bBegin);
        cls.maxManifolds = std::max(cls.maxManifolds, (int32_t)mMembers[gId].size());
        cls.maxJoints = std::max(cls.maxJoints, (int32_t)jMembers[gId].size());
        int32_t gc = 0;
        for (int32_t u : mMembers[gId]) gc = std::max(gc, colour[u] + 1);
        for (int32_t u : jMembers[gId]) gc = std::max(gc, colour[u] + 1);
        std::vector<std::vector<int32_t>> mByColour(gc), jByColour(gc);
        for (int32_t u : jMembers[gId]) jByColour[colour[u]].push_back(u);
        {
            std::vector<std::vector<int32_t>> ms(gc);  // manifolds as list entries, sorted by kind
            for (int32_t u : mMembers[gId]) ms[colour[u]].push_back(u);
            for (int32_t c = 0; c < gc; c++) {
                byKind(ms[c]);
                for (int32_t u : ms[c]) mByColour[c].push_back(u - nj);
                byKind(jByColour[c]);
            }
        }
        d.cCount = gc;
        d.mBegin = slot;
        d.cBegin = (int32_t)plan.colourOffsets.size();
        d.jBegin = jslot;
        d.jcBegin = (int32_t)plan.jointColourOffsets.size();
        for (int32_t c = 0; c < gc; c++) {
            plan.colourOffsets.push_back(slot - d.mBegin);
            plan.jointColourOffsets.push_back(jslot - d.jBegin);
            cls.maxColourMembers = std::max(
                cls.maxColourMembers, (int32_t)std::max(mByColour[c].size(), jByColour[c].size()));
            for (int32_t i : mByColour[c]) {
                plan.slotOf[i] = slot;
                plan.groupOfManifold[i] = k;
                plan.refs[slot] = make_int2(ref(a[nj + i]), ref(b[nj + i]));
                slot++;
            }
            for (int32_t u : jByColour[c]) {
                plan.jointSlotOf[u] = jslot;
                plan.jointRefs[jslot] = make_int2(ref(a[u]), ref(b[u]));
                jslot++;
            }
        }
        plan.colourOffsets.push_back(slot - d.mBegin);
        plan.jointColourOffsets.push_back(jslot - d.jBegin);
        d.mEnd = slot;
        d.jEnd = jslot;
        if (d.jEnd > d.jBegin) plan.groupJoints = true;
    }
}

bepugpu_status Scene::UploadGroups(Context* ctx) {
    const GroupPlan& g = groupPlan;
    size_t G = g.groups.size();
    if (G == 0) return BEPUGPU_OK;
    cudaError_t e;
    if ((e = cudaMemcpyAsync(groupDescDev, g.groups.data(), sizeof(GroupDesc) * G, cudaMemcpyHostToDevice, stream)) ||
        (e = cudaMemcpyAsync(groupBodiesDev, g.groupBodies.data(), sizeof(int32_t) * g.groupBodies.size(),
                             cudaMemcpyHostToDevice, stream)) ||
        (e = cudaMemcpyAsync(groupRefsDev, g.refs.data(), sizeof(int2) * g.refs.size(), cudaMemcpyHostToDevice,
                             stream)) ||
        (e = cudaMemcpyAsync(groupColourOffsetsDev, g.colourOffsets.data(), sizeof(int32_t) * g.colourOffsets.size(),
                             cudaMemcpyHostToDevice, stream)) ||
        (!g.jointRefs.empty() &&
         (e = cudaMemcpyAsync(groupJointRefsDev, g.jointRefs.data(), sizeof(int2) * g.jointRefs.size(),
                              cudaMemcpyHostToDevice, stream))) ||
        (e = cudaMemcpyAsync(groupJointColourOffsetsDev, g.jointColourOffsets.data(),
                             sizeof(int32_t) * g.jointColourOffsets.size(), cudaMemcpyHostToDevice, stream)) ||
        (e = cudaStreamSynchronize(stream))) {
        ctx->SetError("group tables: %s", cudaGetErrorString(e));
        return BEPUGPU_CUDA_ERROR;
    }
    return BEPUGPU_OK;
}

namespace {
int ClassThreads(const GroupClass& c, int override_) {
    if (override_ > 0) return override_;
    int t = ((c.maxColourMembers + 31) / 32) * 32;
    return std::min(std::max(t, 32), 256);
}

template <bool kShared, int kJoints>
bepugpu_status LaunchClass(Context* ctx, Scene* s, const GroupClass& c, const StepParams& p, uint32_t flags,
                           bool count, GroupTables t, bool prestepped, int* launches) {
    if (c.end <= c.begin) return BEPUGPU_OK;
    const int Bc = std::max(c.maxLocal, 1), Lc = std::max(c.maxManifolds, 1), Jc = std::max(c.maxJoints, 1);
    const bool nonConvex = s->groupPlan.nonConvexLanes;
    size_t smemBytes = GroupSmemBytes(kShared, Bc, Lc, kJoints ? Jc : 0, nonConvex);
    cudaError_t e = cudaSuccess;
    if (smemBytes > 48 * 1024) {
        e = cudaFuncSetAttribute(k_groups<false, kShared, kJoints>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smemBytes);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_groups<true, kShared, kJoints>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smemBytes);
        if (e != cudaSuccess) {
            ctx->SetError("group kernel shared memory %zu bytes: %s", smemBytes, cudaGetErrorString(e));
            return BEPUGPU_CUDA_ERROR;
        }
    }
    const int threads = ClassThreads(c, s->groupThreadsOverride);
    const unsigned blocks = (unsigned)(c.end - c.begin);
    // the thread's last error must be this launch's own
    const cudaError_t earlier = cudaGetLastError();
    if (count)
        k_groups<true, kShared, kJoints><<<blocks, threads, smemBytes, s->stream>>>(
            s->m, s->b, s->j, p, flags, t, c.begin, Bc, Lc, Jc, s->Census(), nonConvex, prestepped);
    else
        k_groups<false, kShared, kJoints><<<blocks, threads, smemBytes, s->stream>>>(
            s->m, s->b, s->j, p, flags, t, c.begin, Bc, Lc, Jc, nullptr, nonConvex, prestepped);
    if (launches) (*launches)++;
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        ctx->SetError("group kernel launch (%u CTAs of %d threads, %zu bytes of shared memory): %s%s%s", blocks,
                      threads, smemBytes, cudaGetErrorString(e), earlier != cudaSuccess ? "; earlier error: " : "",
                      earlier != cudaSuccess ? cudaGetErrorString(earlier) : "");
        return BEPUGPU_CUDA_ERROR;
    }
    return BEPUGPU_OK;
}
}  // namespace

bool SplitGroupPrologue(const Scene* s, uint32_t flags) {
    const GroupPlan& g = s->groupPlan;
    if (g.groups.empty() || !(flags & BEPUGPU_STEP_SOLVE)) return false;
    if (s->groupPrologue >= 0) return s->groupPrologue == 1;
    const int32_t held = (g.groups.back().mEnd - g.globalCount) + (g.groups.back().jEnd - g.jointGlobalCount);
    return g.groupJoints && held >= kSplitPrologueConstraints;
}

bepugpu_status LaunchGroups(Context* ctx, Scene* s, const StepParams& p, uint32_t flags, bool count, int* launches) {
    const GroupPlan& g = s->groupPlan;
    if (g.groups.empty()) return BEPUGPU_OK;
    GroupTables t;
    t.groups = s->groupDescDev;
    t.bodies = s->groupBodiesDev;
    t.refs = s->groupRefsDev;
    t.colourOffsets = s->groupColourOffsetsDev;
    t.jointRefs = s->groupJointRefsDev;
    t.jointColourOffsets = s->groupJointColourOffsetsDev;
    const bool split = SplitGroupPrologue(s, flags);
    if (split) {
        // every group's manifold slots follow the sweep part's; its bodies are the body list
        const int s0 = g.globalCount, s1 = g.groups.back().mEnd, nb = g.groups.back().bEnd;
        const int T = 128;
        const cudaError_t earlier = cudaGetLastError();
        if (s1 - s0 + nb > 0)
            k_group_refresh_force<<<(s1 - s0 + nb + T - 1) / T, T, 0, s->stream>>>(s->m, s->b, p, t.bodies, nb, s0,
                                                                                    s1, flags);
        if (s1 > s0) k_group_prestep<<<(s1 - s0 + T - 1) / T, T, 0, s->stream>>>(s->m, s->b, p, s0, s1);
        if (launches) *launches += (s1 - s0 + nb > 0) + (s1 > s0);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            ctx->SetError("group prologue launch: %s%s%s", cudaGetErrorString(e),
                          earlier != cudaSuccess ? "; earlier error: " : "",
                          earlier != cudaSuccess ? cudaGetErrorString(earlier) : "");
            return BEPUGPU_CUDA_ERROR;
        }
    }
    bepugpu_status st = LaunchClass<true, false>(ctx, s, g.shared, p, flags, count, t, split, launches);
    if (st == BEPUGPU_OK) st = LaunchClass<false, false>(ctx, s, g.global, p, flags, count, t, split, launches);
    if (s->addedJointTypes) {
        if (st == BEPUGPU_OK) st = LaunchClass<true, 2>(ctx, s, g.sharedJoints, p, flags, count, t, split, launches);
        if (st == BEPUGPU_OK) st = LaunchClass<false, 2>(ctx, s, g.globalJoints, p, flags, count, t, split, launches);
    } else {
        if (st == BEPUGPU_OK) st = LaunchClass<true, 1>(ctx, s, g.sharedJoints, p, flags, count, t, split, launches);
        if (st == BEPUGPU_OK) st = LaunchClass<false, 1>(ctx, s, g.globalJoints, p, flags, count, t, split, launches);
    }
    return st;
}

}  // namespace bepugpu
